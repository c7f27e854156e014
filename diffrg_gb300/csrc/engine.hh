// engine.hh -- host-side internals of libgbint (context, provider caches, node pool, batches).
#pragma once

#include <atomic>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "engine_types.hh"
#include "gbint.h"
#include "host_quadrature.hh"

namespace gbint
{
  // cache key of one quadrature axis (kind + order + the parameters its nodes depend on)
  struct AxisKey {
    int kind = 0;
    int n = 0;
    double p[7] = {0, 0, 0, 0, 0, 0, 0};
    bool operator<(const AxisKey &o) const
    {
      if (kind != o.kind) return kind < o.kind;
      if (n != o.n) return n < o.n;
      return std::memcmp(p, o.p, sizeof(p)) < 0;
    }
  };

  struct HostAxis {
    std::vector<double> v, w, a;
    int pm_from = 1 << 30;
  };

  struct GLRule {
    std::vector<double> x, w;
    double *d64x = nullptr, *d64w = nullptr;
    float *d32x = nullptr, *d32w = nullptr;
  };
  struct MatsEntry {
    double T, E;
    MatsRule rule;
    double *d64x = nullptr, *d64w = nullptr;
    float *d32x = nullptr, *d32w = nullptr;
  };

  // device pool of axis nodes (FP64 arrays + 32-byte FP32 records).  An axis keeps its offset
  // while any batch holds it; unheld axes are evicted (their ranges go to the free list) only
  // when an allocation would otherwise fail.
  struct NodePool {
    int capacity = 0, used = 0;
    double *d_v = nullptr, *d_w = nullptr, *d_a = nullptr;
    NodeRec *d_rec = nullptr;
    std::map<int, int> free_ranges;  // offset -> length
    uint64_t evictions = 0;
  };

  struct AxisEntry {
    AxisRef ref;
    int refs = 0;           // batches (and in-progress calls) holding the axis
    std::vector<double> v;  // host copy of the node values
    std::vector<double> w;  // host copy of the weights
  };

  struct Ticket;
  struct ServeState;
  struct DLoopState;
  struct SlotPool;
} // namespace gbint

struct gb_table {
  int slot = -1;
  gb_table_spec spec{};
  float *buf[2] = {nullptr, nullptr};
  int front = 0;
  uint64_t epoch = 0;
  int elems = 0;
  int bytes = 0;  // padded to 16
};

struct gb_batch {
  int n = 0;
  int precision = GB_PREC_FP32C;
  std::vector<gb_integral> src;
  std::vector<gbint::ItemDev> items;
  std::vector<gbint::UnitDev> units;       // host-built units (cost-ordered runs only)
  std::vector<gbint::ExpandDev> expand;    // per-integral unit ranges, expanded on the device
  size_t n_units_total = 0;
  bool host_units = false;
  std::vector<gbint::SegDev> segs;
  std::vector<float4> aux;  // per-item constants (S kinds)
  struct KindRun {
    int kind = 0;
    int unit_begin = 0, n_units = 0;
    int threads = 0, ctas = 0, tab_cap = 0, rec_cap = 0;
  };
  std::vector<KindRun> runs;
  std::vector<int> plain_loop_axis;
  std::vector<long long> plain_threads;
  int seg_max_entries = 0;
  size_t seg_total = 0;
  uint64_t points = 0;
  // device
  gbint::ItemDev *d_items = nullptr;
  gbint::UnitDev *d_units = nullptr;
  gbint::ExpandDev *d_expand = nullptr;
  gbint::SegDev *d_segs = nullptr;
  double *d_seg = nullptr;
  float4 *d_aux = nullptr;
  double *d_partials = nullptr;
  int *d_item_count = nullptr;
  int *d_counters = nullptr;  // one per kind run
  double *d_out = nullptr;
  int *h_err = nullptr;  // pinned landing place of the context's error word (gb_batch_results)
  size_t bytes = 0;
  // graph replay
  cudaGraphExec_t graph = nullptr;
  cudaStream_t graph_stream = nullptr;
  // axes held in the node pool while the batch exists
  std::vector<gbint::AxisKey> held;
  bool arena = false;  // device buffers belong to a serving slot (not freed with the batch)
  bool single = false;  // one CTA per work unit, each evaluating its own unit (serving)
};

struct gb_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::vector<cudaStream_t> pool_streams;
  std::recursive_mutex mu;
  size_t budget = 0;
  std::atomic<size_t> in_use{0};
  std::string last_error;
  // provider
  int mats_min = 32, mats_vacuum = 48, mats_add = 0;
  std::map<int, gbint::GLRule> gl;
  std::map<std::pair<int, int>, gbint::GLRule> rules;  // (QuadratureType, order), types other than Legendre
  std::vector<std::unique_ptr<gbint::MatsEntry>> mats;
  // nodes
  gbint::NodePool pool;
  std::map<gbint::AxisKey, gbint::AxisEntry> axis_cache;
  // tables
  gbint::TableDev *d_dir = nullptr;
  std::vector<gbint::TableDev> h_dir;
  std::vector<gb_table *> slots;
  cudaEvent_t tables_event = nullptr;  // recorded after every table update (serving orders on it)
  int update_depth = 0;                // open gb_table_group_begin blocks (guarded by mu)
  int *d_err = nullptr;
  // work-unit schedule per FP32-compensated kind (autotuner; zero fields = defaults),
  // indexed by kind slot = base kind + 8 * accurate
  gb_schedule sched[16] = {};
  std::string tune_report;  // JSON of the last gb_autotune's measurements
  // plain-path scratch
  std::vector<double *> plain_buf;
  std::vector<size_t> plain_buf_elems;
  std::vector<void *> plain_tmp;
  std::vector<size_t> plain_tmp_bytes;
  double *plain_res = nullptr;     // device, per stream
  double *plain_res_h = nullptr;   // pinned host
  // serving
  gbint::ServeState *serve = nullptr;
  // device-resident request loop (dloop.cu), the other serving mode
  gbint::DLoopState *dloop = nullptr;
  // request slots of the C++ class templates
  gbint::SlotPool *slotpool = nullptr;
  // gb_buffer_* allocations and their sizes
  std::map<void *, size_t> buffers;
};

namespace gbint
{
  int set_error(gb_ctx *ctx, int code, const std::string &msg);
  int cuda_fail(gb_ctx *ctx, cudaError_t e, const char *what);
  int build_batch(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
                  gb_batch **out);
  // host half of build_batch: descriptors, units, segments, kind runs; item i reads the
  // tables item_tables[i][0..item_ntables[i]).  Caller holds ctx->mu; b->held keeps the axes.
  int plan_batch(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *const *item_tables,
                 const int *item_ntables, int precision, gb_batch *b);
  size_t batch_device_bytes(const gb_batch *b);
  // the schedule plan_batch uses for an FP32-compensated kind, defaults filled in
  gb_schedule resolve_schedule(const gb_ctx *ctx, int kind);
  void release_axes(gb_ctx *ctx, std::vector<AxisKey> &held);
  // the table-update stream waits for in-flight serving batches (double-buffer reuse)
  int serve_fence_tables(gb_ctx *ctx, cudaStream_t s);
  int run_batch(gb_ctx *ctx, gb_batch *b, double *d_out, cudaStream_t s);
  void free_batch(gb_ctx *ctx, gb_batch *b);
  // serving
  int serve_start(gb_ctx *ctx, int max_inflight, int max_items);
  int serve_stop(gb_ctx *ctx);
  int serve_submit(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
                   gb_ticket *out);
  int serve_poll(gb_ctx *ctx, gb_ticket t, double *out, bool wait, double timeout_s);
  int serve_cancel(gb_ctx *ctx, gb_ticket t);
  int serve_stats(gb_ctx *ctx, gb_stats *out);
  int serve_reset_stats(gb_ctx *ctx);
  // device-resident request loop
  int dloop_start(gb_ctx *ctx, int ring_slots, int max_items, long long max_units, double idle_s);
  int dloop_stop(gb_ctx *ctx);
  int dloop_fence_tables(gb_ctx *ctx);
  int dloop_submit(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
                   gb_ticket *out);
  int dloop_poll(gb_ctx *ctx, gb_ticket t, double *out, bool wait, double timeout_s);
  int dloop_stats(gb_ctx *ctx, gb_stats *out);
  int dloop_reset_stats(gb_ctx *ctx);
  int dloop_info(gb_ctx *ctx, long long *launches, int *idle_exits, int *running);
  void destroy_slots(gb_ctx *ctx);
} // namespace gbint

// return the CUDA failure (with the failing call's text) from a function that has `ctx`
#define GB_CUDA(call)                                           \
  do {                                                          \
    cudaError_t e__ = (call);                                   \
    if (e__ != cudaSuccess) return gbint::cuda_fail(ctx, e__, #call); \
  } while (0)
