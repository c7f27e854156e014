// dloop.cu -- the device-resident request loop (gb_serve_start_device).
//
// A second serving mode beside the host dispatcher of serve.cc.  gb_submit writes a request
// straight into a ring the GPU reads: its integral descriptors (the FP64 items of gb_get), a
// snapshot of its tables' directory entries and its work-unit range go into the request's ring
// slot in device memory (one stream-ordered copy), then the request is published by raising the
// count of published work units in mapped host memory.  A persistent kernel (one CTA of 256
// threads per SM, so other kernels still find room) claims published units one at a time with
// an atomic compare-and-swap on a device counter -- continuous batching: units of a request that
// arrives while others run are claimed as soon as CTAs free up, and requests of different sizes
// and integrand kinds share the launch.  Requests of at most 2^22 grid points are published on
// an express lane whose units CTAs claim first, so a small request arriving behind a large one
// starts as soon as CTAs finish their current units.  A unit is 1024 grid points of one integral, evaluated
// with the same per-point function and reduction as the generic FP64 kernel; the last unit of an
// integral to arrive sums the integral's unit partials in unit order, so every result is
// bit-identical alone and in any mix, and equals gb_get(..., GB_PREC_FP64) to rounding (the
// same function and order, compiled into another kernel).  Results and a per-request
// done flag go to mapped host memory.  A watcher thread reads the done flags every 20 us while
// requests are outstanding (it sleeps otherwise): it stamps each request's completion (latency =
// submit -> results in host memory), frees its ring slot, and relaunches the kernel when work is
// published but no loop runs; gb_poll / gb_wait then find the results without a CUDA call.
//
// Every wait is bounded.  A CTA that finds no published work polls with a clock64 budget (the
// idle time given at start) and an iteration cap, then counts an idle exit and leaves; the host
// relaunches the kernel when a request is published, or (the watcher) when a request was
// published just as the last CTA left.  The loop
// also leaves (and is relaunched fresh) around table updates and after the node pool recycled
// storage, so no CTA keeps stale L1 lines of a table buffer or node range the host rewrote.
//
// Admission by memory: the ring has a fixed number of slots, each with device room for
// max_items integrals and max_units work units, allocated at start and counted against the
// context's HBM budget.  A request waits for its slot to free (the request published R slots
// earlier has been collected); one that can never fit is refused with GB_EBUDGET.
// Table updates wait for every published request to finish before they write (each request
// reads one epoch of every table).  Requests are evaluated in FP64 whatever precision they ask.
#include "device_common.cuh"
#include "engine.hh"
#include "integrands.cuh"
#include "kernels.hh"

#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdint>
#include <cstring>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <thread>

namespace gbint
{
  int prepare_item_fp64(gb_ctx *ctx, const gb_integral &g, gb_table *const *tables, int n_tables, ItemDev &it,
                        uint64_t &grid_points, std::vector<AxisKey> &hold);

  namespace
  {
    constexpr int kDLMaxRing = 64;
    // requests of at most this many grid points go to the express lane, whose units the loop's
    // CTAs claim before the normal lane's: a small request does not wait behind the units of a
    // large one that arrived first
    constexpr uint64_t kDLExpressPoints = 1ull << 22;
    constexpr int kDLMaxTables = kMaxTables;  // distinct tables one request may read (the whole directory)

    // a ring slot's request, in device memory (pointers as integers: read with ld.global.cg)
    struct DLReq {
      long long u_begin, u_end;  // its work units, numbered within its lane
      int n_items, seq, lane, pad;
      unsigned long long items, tabs, partials, item_count, done_items;
    };
    struct DLShared {  // device memory
      unsigned long long next_unit[2];  // per lane: 0 normal, 1 express
      int idle_exits;
      int pad;
    };
    struct DLMapped {  // mapped pinned host memory
      volatile unsigned long long published[2];  // per lane
      volatile int stop;
      volatile int pad0;
      volatile int done[kDLMaxRing];  // seq of the last finished request of each slot
    };
    struct DLParams {
      const DLReq *reqs;
      int R, max_items;
      DLShared *sh;
      DLMapped *m;      // device address of the mapped block
      double *results;  // device address of the mapped results, [R][max_items]
      const double *pv, *pw;
      long long idle_cycles;
      int max_polls;
      int *err;
    };

    __device__ __forceinline__ void ldcg_words(int *dst, const int *src, int words, int tid, int nt)
    {
      for (int i = tid; i < words; i += nt) dst[i] = __ldcg(src + i);
    }

    __global__ void __launch_bounds__(kGenericThreads) k_dloop(const DLParams L)
    {
      __shared__ double red[32];
      __shared__ long long s_u;
      __shared__ int s_slot, s_item, s_flag;
      __shared__ long long s_ub;
      __shared__ int s_nitems, s_seq;
      __shared__ unsigned long long s_items, s_tabs, s_partials, s_count, s_done;
      __shared__ __align__(16) ItemDev s_it;
      __shared__ __align__(16) TableDev sT[4];
      int hint = 0;
      for (;;) {
        if (threadIdx.x == 0) {
          long long u = -1;
          int lane = 0;
          int polls = 0;
          long long t0 = 0;
          for (;;) {
            const unsigned long long pub1 = L.m->published[1], pub0 = L.m->published[0];
            __threadfence_system();
            // the express lane first
            const unsigned long long n1 = atomicAdd(&L.sh->next_unit[1], 0ull);
            if (n1 < pub1) {
              if (atomicCAS(&L.sh->next_unit[1], n1, n1 + 1) == n1) {
                u = (long long)n1;
                lane = 1;
                break;
              }
              continue;
            }
            const unsigned long long n0 = atomicAdd(&L.sh->next_unit[0], 0ull);
            if (n0 < pub0) {
              if (atomicCAS(&L.sh->next_unit[0], n0, n0 + 1) == n0) {
                u = (long long)n0;
                lane = 0;
                break;
              }
              continue;
            }
            if (L.m->stop) break;
            if (polls == 0) t0 = clock64();
            if (++polls > L.max_polls || clock64() - t0 > L.idle_cycles) {
              atomicAdd(&L.sh->idle_exits, 1);
              break;
            }
            __nanosleep(2000);  // idle: about one read of the host's counter per 2 us per CTA
          }
          int slot = -1;
          if (u >= 0) {
            for (int k = 0; k < L.R; ++k) {
              const int s = (hint + k) % L.R;
              const long long b = __ldcg(&L.reqs[s].u_begin), e = __ldcg(&L.reqs[s].u_end);
              if (u >= b && u < e && __ldcg(&L.reqs[s].lane) == lane) {
                slot = s;
                break;
              }
            }
            if (slot >= 0) {
              hint = slot;
              const DLReq *r = L.reqs + slot;
              s_ub = __ldcg(&r->u_begin);
              s_nitems = __ldcg(&r->n_items);
              s_seq = __ldcg(&r->seq);
              s_items = __ldcg(&r->items);
              s_tabs = __ldcg(&r->tabs);
              s_partials = __ldcg(&r->partials);
              s_count = __ldcg(&r->item_count);
              s_done = __ldcg(&r->done_items);
              // the unit's integral: items sorted by their first unit
              const ItemDev *items = reinterpret_cast<const ItemDev *>(s_items);
              const int lu = (int)(u - s_ub);
              int lo = 0, hi = s_nitems - 1;
              while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (__ldcg(&items[mid].unit_begin) <= lu)
                  lo = mid;
                else
                  hi = mid - 1;
              }
              s_item = lo;
            } else
              atomicOr(L.err, kErrBadIndex);  // a claimed unit in no published request: recorded, skipped
          }
          s_u = u;
          s_slot = slot;
        }
        __syncthreads();
        const long long u = s_u;
        if (u < 0) break;
        if (s_slot < 0) {
          __syncthreads();
          continue;
        }
        const int slot = s_slot, item = s_item;
        // the integral's descriptor and its tables (rewritten by the host per request: read past L1)
        ldcg_words(reinterpret_cast<int *>(&s_it),
                   reinterpret_cast<const int *>(reinterpret_cast<const ItemDev *>(s_items) + item),
                   (int)(sizeof(ItemDev) / 4), threadIdx.x, blockDim.x);
        __syncthreads();
        const TableDev *tabs = reinterpret_cast<const TableDev *>(s_tabs);
        for (int t = 0; t < 4; ++t)
          if (s_it.tab[t] >= 0)
            ldcg_words(reinterpret_cast<int *>(&sT[t]), reinterpret_cast<const int *>(tabs + s_it.tab[t]),
                       (int)(sizeof(TableDev) / 4), threadIdx.x, blockDim.x);
        __syncthreads();
        const ItemDev &it = s_it;
        const int lu = (int)(u - s_ub);
        const long long begin = (long long)(lu - it.unit_begin) * kGenericUnitPoints;
        const long long count = min((long long)kGenericUnitPoints, (long long)it.rows - begin);
        double acc = 0.0;
#pragma unroll 1
        for (int k = 0; k < kGenericPPT; ++k) {
          const int local = threadIdx.x + k * blockDim.x;
          if (local < count) acc += dev::eval_point_fp64(it, begin + local, L.pv, L.pw, sT);
        }
        const double tot = dev::block_sum(acc, red);
        double *partials = reinterpret_cast<double *>(s_partials);
        int *item_count = reinterpret_cast<int *>(s_count);
        if (threadIdx.x == 0) {
          partials[lu] = tot;
          __threadfence();
          s_flag = (atomicAdd(&item_count[item], 1) == it.n_units - 1);
        }
        __syncthreads();
        if (s_flag) {  // the integral's unit partials in unit order (as the generic kernel's finish)
          __threadfence();
          double v = 0.0;
          for (int i = threadIdx.x; i < it.n_units; i += blockDim.x) v += __ldcg(&partials[it.unit_begin + i]);
          v = dev::block_sum(v, red);
          if (threadIdx.x == 0) {
            L.results[(size_t)slot * L.max_items + item] = it.args[0] + v;
            item_count[item] = 0;
            __threadfence_system();  // the result (host memory) before this integral counts as done
            int *done_items = reinterpret_cast<int *>(s_done);
            if (atomicAdd(done_items, 1) == s_nitems - 1) {  // the request's last integral
              *done_items = 0;
              __threadfence_system();
              L.m->done[slot] = s_seq;
            }
          }
        }
        __syncthreads();
      }
    }

    double now_s()
    {
      return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
    }

    struct DLSlot {
      // device arena
      DLReq *d_req = nullptr;
      ItemDev *d_items = nullptr;
      TableDev *d_tabs = nullptr;
      double *d_partials = nullptr;
      int *d_count = nullptr;  // item arrival counters, then the request's done counter
      // pinned staging
      DLReq *h_req = nullptr;
      ItemDev *h_items = nullptr;
      TableDev *h_tabs = nullptr;
      bool busy = false;
      int seq = 0;
      gb_ticket ticket = 0;
    };

    struct DLTicket {
      int slot = -1, seq = 0, n = 0;
      double t_submit = 0;
      std::vector<AxisKey> held;
      bool done = false;
      std::vector<double> results;
    };
  } // namespace

  struct DLoopState {
    int R = 16, max_items = 2048;
    long long max_units = 1 << 21;
    double idle_s = 5e-3;
    std::vector<DLSlot> slots;
    char *d_arena = nullptr;
    DLShared *d_shared = nullptr;
    DLReq *d_reqs = nullptr;  // the R slot requests, contiguous (the kernel scans them)
    DLMapped *h_map = nullptr, *d_map = nullptr;
    double *h_results = nullptr, *d_results = nullptr;
    cudaStream_t loop_stream = nullptr, copy_stream = nullptr;
    cudaEvent_t loop_done = nullptr;
    bool launched = false;
    uint64_t evictions_at_launch = 0;
    long long launches = 0;
    unsigned long long published[2] = {0, 0};  // per lane
    int next_seq = 1;
    gb_ticket next_ticket = 1;
    std::map<gb_ticket, DLTicket> tickets;
    size_t bytes = 0;
    int sm_mhz = 2000;
    // statistics
    uint64_t submitted = 0, completed = 0, rejected = 0, points = 0;
    std::vector<double> lat;
    double t_start = 0;
    // completion watcher (guarded by ctx->mu)
    std::thread watcher;
    std::condition_variable_any wake;
    bool stop_watcher = false;
  };

  namespace
  {
    bool loop_running(DLoopState *D)
    {
      if (!D->launched) return false;
      const cudaError_t q = cudaEventQuery(D->loop_done);
      if (q == cudaErrorNotReady) return true;
      D->launched = false;
      return false;
    }

    int launch_loop(gb_ctx *ctx, DLoopState *D)
    {
      DLParams L{};
      L.reqs = D->d_reqs;
      L.R = D->R;
      L.max_items = D->max_items;
      L.sh = D->d_shared;
      L.m = D->d_map;
      L.results = D->d_results;
      L.pv = ctx->pool.d_v;
      L.pw = ctx->pool.d_w;
      L.idle_cycles = (long long)(D->idle_s * D->sm_mhz * 1e6);
      L.max_polls = (int)std::min<double>(1e8, D->idle_s * 5e5 + 100);  // ~ one poll per 2 us of sleep
      L.err = ctx->d_err;
      k_dloop<<<ctx->num_sms, kGenericThreads, 0, D->loop_stream>>>(L);
      cudaError_t e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaEventRecord(D->loop_done, D->loop_stream);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "device request loop launch");
      D->launched = true;
      D->launches++;
      D->evictions_at_launch = ctx->pool.evictions;
      return GB_OK;
    }

    // ask the loop to leave and wait for it (its idle CTAs leave at once; busy ones finish the
    // units they claimed and any claimable ones first)
    int stop_loop(gb_ctx *ctx, DLoopState *D)
    {
      if (!D->launched) return GB_OK;
      D->h_map->stop = 1;
      std::atomic_thread_fence(std::memory_order_seq_cst);
      const cudaError_t e = cudaEventSynchronize(D->loop_done);
      D->h_map->stop = 0;
      std::atomic_thread_fence(std::memory_order_seq_cst);
      D->launched = false;
      if (e != cudaSuccess) return cuda_fail(ctx, e, "device request loop");
      return GB_OK;
    }

    // collect a finished request of the ring (its slot frees); caller holds ctx->mu
    bool reap(gb_ctx *ctx, DLoopState *D, gb_ticket t)
    {
      auto it = D->tickets.find(t);
      if (it == D->tickets.end()) return false;
      DLTicket &k = it->second;
      if (k.done) return true;
      if (D->h_map->done[k.slot] != k.seq) return false;
      std::atomic_thread_fence(std::memory_order_acquire);
      const double *r = D->h_results + (size_t)k.slot * D->max_items;
      k.results.assign(r, r + k.n);
      k.done = true;
      D->lat.push_back(now_s() - k.t_submit);
      D->completed++;
      release_axes(ctx, k.held);
      D->slots[k.slot].busy = false;
      return true;
    }

    // the watcher: reaps finished requests as they finish and keeps a loop running while
    // published work is outstanding
    void watch(gb_ctx *ctx, DLoopState *D)
    {
      cudaSetDevice(ctx->device);
      std::unique_lock<std::recursive_mutex> lk(ctx->mu);
      while (!D->stop_watcher) {
        bool pending = false;
        for (auto &kv : D->tickets)
          if (!kv.second.done && !reap(ctx, D, kv.first)) pending = true;
        if (pending && !loop_running(D)) launch_loop(ctx, D);  // a failure resurfaces at gb_wait
        if (pending) {
          lk.unlock();
          std::this_thread::sleep_for(std::chrono::microseconds(20));
          lk.lock();
        } else {
          D->wake.wait_for(lk, std::chrono::milliseconds(50));
        }
      }
    }

    void free_state(DLoopState *D)
    {
      for (auto &s : D->slots) {
        cudaFreeHost(s.h_req);
        cudaFreeHost(s.h_items);
        cudaFreeHost(s.h_tabs);
      }
      cudaFree(D->d_reqs);
      cudaFree(D->d_arena);
      cudaFree(D->d_shared);
      if (D->h_map) cudaFreeHost(D->h_map);
      if (D->h_results) cudaFreeHost(D->h_results);
      if (D->loop_stream) cudaStreamDestroy(D->loop_stream);
      if (D->copy_stream) cudaStreamDestroy(D->copy_stream);
      if (D->loop_done) cudaEventDestroy(D->loop_done);
    }
  } // namespace

  int dloop_start(gb_ctx *ctx, int ring_slots, int max_items, long long max_units, double idle_s)
  {
    if (!ctx) return GB_EINVAL;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    if (ctx->serve || ctx->dloop) return set_error(ctx, GB_EINVAL, "serving already started");
    if (ring_slots < 1 || ring_slots > kDLMaxRing || max_items < 1 || max_units < 1 || !(idle_s > 0) || idle_s > 10)
      return set_error(ctx, GB_EINVAL,
                       "gb_serve_start_device: ring_slots 1..64, max_items >= 1, max_units >= 1, idle 0..10 s");
    GB_CUDA(cudaSetDevice(ctx->device));
    auto D = std::make_unique<DLoopState>();
    D->R = ring_slots;
    D->max_items = max_items;
    D->max_units = max_units;
    D->idle_s = idle_s;
    int clk_khz = 0;
    if (cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, ctx->device) == cudaSuccess && clk_khz > 0)
      D->sm_mhz = clk_khz / 1000;
    // device arena: per slot items, table snapshot, partials, counters -- one allocation
    const size_t per_items = (size_t)max_items * sizeof(ItemDev), per_tabs = kDLMaxTables * sizeof(TableDev);
    const size_t per_part = (size_t)max_units * sizeof(double), per_cnt = ((size_t)max_items + 1) * sizeof(int);
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t per_slot = al(per_items) + al(per_tabs) + al(per_part) + al(per_cnt);
    const size_t total = per_slot * ring_slots + al(sizeof(DLReq) * ring_slots) + al(sizeof(DLShared));
    if (ctx->in_use + total > ctx->budget)
      return set_error(ctx, GB_EBUDGET, "gb_serve_start_device: the ring does not fit the HBM budget");
    cudaError_t e = cudaSuccess;
    char *arena = nullptr;
    e = cudaMalloc(&arena, per_slot * ring_slots);
    if (e == cudaSuccess) D->d_arena = arena;
    if (e == cudaSuccess) e = cudaMemset(arena, 0, per_slot * ring_slots);
    if (e == cudaSuccess) e = cudaMalloc(&D->d_reqs, sizeof(DLReq) * ring_slots);
    if (e == cudaSuccess) e = cudaMemset(D->d_reqs, 0, sizeof(DLReq) * ring_slots);
    if (e == cudaSuccess) e = cudaMalloc(&D->d_shared, sizeof(DLShared));
    if (e == cudaSuccess) e = cudaMemset(D->d_shared, 0, sizeof(DLShared));
    if (e == cudaSuccess) e = cudaHostAlloc(&D->h_map, sizeof(DLMapped), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&D->d_map, D->h_map, 0);
    if (e == cudaSuccess)
      e = cudaHostAlloc(&D->h_results, (size_t)ring_slots * max_items * sizeof(double), cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&D->d_results, D->h_results, 0);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&D->loop_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&D->copy_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&D->loop_done, cudaEventDisableTiming);
    D->slots.resize(ring_slots);
    for (int s = 0; s < ring_slots && e == cudaSuccess; ++s) {
      DLSlot &sl = D->slots[s];
      char *p = arena + per_slot * s;
      sl.d_items = reinterpret_cast<ItemDev *>(p);
      sl.d_tabs = reinterpret_cast<TableDev *>(p + al(per_items));
      sl.d_partials = reinterpret_cast<double *>(p + al(per_items) + al(per_tabs));
      sl.d_count = reinterpret_cast<int *>(p + al(per_items) + al(per_tabs) + al(per_part));
      sl.d_req = D->d_reqs + s;
      e = cudaMallocHost(&sl.h_req, sizeof(DLReq));
      if (e == cudaSuccess) e = cudaMallocHost(&sl.h_items, per_items);
      if (e == cudaSuccess) e = cudaMallocHost(&sl.h_tabs, per_tabs);
    }
    if (e != cudaSuccess) {
      free_state(D.get());
      return cuda_fail(ctx, e, "gb_serve_start_device");
    }
    std::memset((void *)D->h_map, 0, sizeof(DLMapped));
    D->bytes = total;
    ctx->in_use += total;
    D->t_start = now_s();
    ctx->dloop = D.release();
    ctx->dloop->watcher = std::thread(watch, ctx, ctx->dloop);
    return GB_OK;
  }

  int dloop_stop(gb_ctx *ctx)
  {
    if (!ctx || !ctx->dloop) return GB_OK;
    DLoopState *D = ctx->dloop;
    {
      std::lock_guard<std::recursive_mutex> lk(ctx->mu);
      D->stop_watcher = true;
      D->wake.notify_all();
    }
    if (D->watcher.joinable()) D->watcher.join();
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    // published requests finish first (the loop is relaunched for them if it left)
    const double deadline = now_s() + 30.0;
    for (auto &kv : D->tickets)
      while (!kv.second.done && D->h_map->done[kv.second.slot] != kv.second.seq && now_s() < deadline) {
        if (!loop_running(D)) launch_loop(ctx, D);
        std::this_thread::sleep_for(std::chrono::microseconds(50));
      }
    stop_loop(ctx, D);
    for (auto &kv : D->tickets) release_axes(ctx, kv.second.held);
    ctx->in_use -= D->bytes;
    free_state(D);
    delete D;
    ctx->dloop = nullptr;
    return GB_OK;
  }

  // a table update writes a buffer published requests may read: they finish first, and the loop
  // leaves so that the next one starts with no cached lines of the old data
  int dloop_fence_tables(gb_ctx *ctx)
  {
    DLoopState *D = ctx->dloop;
    const double deadline = now_s() + 30.0;
    for (auto &kv : D->tickets) {
      while (!reap(ctx, D, kv.first)) {
        if (now_s() > deadline) return set_error(ctx, GB_ETIMEDOUT, "table update: device-loop requests did not finish");
        if (!loop_running(D)) {
          const int rc = launch_loop(ctx, D);
          if (rc) return rc;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(20));
      }
    }
    return stop_loop(ctx, D);
  }

  int dloop_submit(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables, int precision,
                   gb_ticket *out)
  {
    (void)precision;  // evaluated in FP64
    if (!items || n <= 0 || !out || n_tables < 0 || (n_tables > 0 && !tables))
      return set_error(ctx, GB_EINVAL, "gb_submit: bad arguments");
    DLoopState *D = ctx->dloop;
    if (n > D->max_items) {
      std::lock_guard<std::recursive_mutex> lk(ctx->mu);
      D->rejected++;
      return set_error(ctx, GB_EBUDGET, "request has more integrals than a device-loop slot holds (max_items)");
    }
    const double t_submit = now_s();
    // the slot of this request frees when the request R submissions earlier is collected; a
    // table-update group that is open finishes first (the request sees all of it or none)
    std::unique_lock<std::recursive_mutex> lk(ctx->mu);
    for (;;) {
      const int s = (D->next_seq - 1) % D->R;
      if (D->slots[s].busy) reap(ctx, D, D->slots[s].ticket);
      if (!D->slots[s].busy && ctx->update_depth == 0) break;
      if (D->slots[s].busy && !loop_running(D)) {
        const int rc = launch_loop(ctx, D);
        if (rc) return rc;
      }
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(20));
      lk.lock();
    }
    GB_CUDA(cudaSetDevice(ctx->device));
    const int s = (D->next_seq - 1) % D->R;
    DLSlot &sl = D->slots[s];
    DLTicket k;
    k.slot = s;
    k.n = n;
    k.t_submit = t_submit;
    // descriptors: the FP64 items of gb_get, their tables remapped onto the request's snapshot
    std::vector<int> dir_slots;
    long long units = 0;
    uint64_t pts = 0;
    for (int i = 0; i < n; ++i) {
      ItemDev it;
      uint64_t points = 0;
      int rc = prepare_item_fp64(ctx, items[i], tables, n_tables, it, points, k.held);
      if (rc) {
        release_axes(ctx, k.held);
        return rc;
      }
      for (int t = 0; t < 4; ++t) {
        if (it.tab[t] < 0) continue;
        auto f = std::find(dir_slots.begin(), dir_slots.end(), it.tab[t]);
        if (f == dir_slots.end()) {
          if ((int)dir_slots.size() == kDLMaxTables) {
            release_axes(ctx, k.held);
            D->rejected++;
            return set_error(ctx, GB_EINVAL, "a device-loop request reads more distinct tables than the directory holds");
          }
          dir_slots.push_back(it.tab[t]);
          f = dir_slots.end() - 1;
        }
        it.tab[t] = (int)(f - dir_slots.begin());
      }
      if (points > (uint64_t)INT32_MAX) {
        release_axes(ctx, k.held);
        D->rejected++;
        return set_error(ctx, GB_EBUDGET, "an integral of more than 2^31 grid points does not fit a device-loop slot");
      }
      it.kind = K_GENERIC;
      it.rows = (int)points;
      it.n_units = (int)((points + kGenericUnitPoints - 1) / kGenericUnitPoints);
      it.unit_begin = (int)units;
      units += it.n_units;
      pts += points;
      if (units > D->max_units) {
        release_axes(ctx, k.held);
        D->rejected++;
        return set_error(ctx, GB_EBUDGET, "request has more work units than a device-loop slot holds (max_units)");
      }
      sl.h_items[i] = it;
    }
    for (size_t t = 0; t < dir_slots.size(); ++t) sl.h_tabs[t] = ctx->h_dir[dir_slots[t]];
    // the tables' last update has landed; a loop that may hold stale lines of recycled node
    // storage is replaced
    cudaError_t e = cudaEventSynchronize(ctx->tables_event);
    if (e != cudaSuccess) {
      release_axes(ctx, k.held);
      return cuda_fail(ctx, e, "gb_submit: table update");
    }
    if (D->launched && ctx->pool.evictions != D->evictions_at_launch) {
      const int rc = stop_loop(ctx, D);
      if (rc) {
        release_axes(ctx, k.held);
        return rc;
      }
    }
    DLReq &r = *sl.h_req;
    const int lane = pts <= kDLExpressPoints ? 1 : 0;
    r.u_begin = (long long)D->published[lane];
    r.u_end = r.u_begin + units;
    r.n_items = n;
    r.seq = D->next_seq;
    r.lane = lane;
    r.items = reinterpret_cast<unsigned long long>(sl.d_items);
    r.tabs = reinterpret_cast<unsigned long long>(sl.d_tabs);
    r.partials = reinterpret_cast<unsigned long long>(sl.d_partials);
    r.item_count = reinterpret_cast<unsigned long long>(sl.d_count);
    r.done_items = reinterpret_cast<unsigned long long>(sl.d_count + D->max_items);
    e = cudaMemcpyAsync(sl.d_items, sl.h_items, n * sizeof(ItemDev), cudaMemcpyHostToDevice, D->copy_stream);
    if (e == cudaSuccess && !dir_slots.empty())
      e = cudaMemcpyAsync(sl.d_tabs, sl.h_tabs, dir_slots.size() * sizeof(TableDev), cudaMemcpyHostToDevice,
                          D->copy_stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sl.d_req, sl.h_req, sizeof(DLReq), cudaMemcpyHostToDevice, D->copy_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(D->copy_stream);
    if (e != cudaSuccess) {
      release_axes(ctx, k.held);
      return cuda_fail(ctx, e, "gb_submit: device-loop descriptors");
    }
    // publish: the descriptors are in device memory before the unit count the loop polls rises
    std::atomic_thread_fence(std::memory_order_seq_cst);
    D->published[lane] = (unsigned long long)r.u_end;
    D->h_map->published[lane] = D->published[lane];
    std::atomic_thread_fence(std::memory_order_seq_cst);
    k.seq = D->next_seq++;
    const gb_ticket id = D->next_ticket++;
    sl.busy = true;
    sl.seq = k.seq;
    sl.ticket = id;
    D->tickets.emplace(id, std::move(k));
    D->submitted++;
    D->points += pts;
    if (!loop_running(D)) {
      const int rc = launch_loop(ctx, D);
      if (rc) return rc;
    }
    D->wake.notify_all();
    *out = id;
    return GB_OK;
  }

  int dloop_poll(gb_ctx *ctx, gb_ticket t, double *out, bool wait, double timeout_s)
  {
    DLoopState *D = ctx->dloop;
    const double deadline = now_s() + (timeout_s > 0 ? timeout_s : 1e9);
    std::unique_lock<std::recursive_mutex> lk(ctx->mu);
    if (!D->tickets.count(t)) return set_error(ctx, GB_EINVAL, "unknown ticket");
    for (;;) {
      if (reap(ctx, D, t)) break;
      // published work and no loop: the loop left while the request was in flight -- relaunch
      if (!loop_running(D)) {
        const int rc = launch_loop(ctx, D);
        if (rc) return rc;
      }
      if (!wait) return GB_EAGAIN;
      if (now_s() > deadline) return set_error(ctx, GB_ETIMEDOUT, "gb_wait timed out");
      lk.unlock();
      std::this_thread::sleep_for(std::chrono::microseconds(5));
      lk.lock();
    }
    auto it = D->tickets.find(t);
    if (out) std::copy(it->second.results.begin(), it->second.results.end(), out);
    D->tickets.erase(it);
    return GB_OK;
  }

  int dloop_stats(gb_ctx *ctx, gb_stats *out)
  {
    DLoopState *D = ctx->dloop;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    out->submitted = D->submitted;
    out->completed = D->completed;
    out->rejected = D->rejected;
    out->batches_launched = (uint64_t)D->launches;
    out->points_evaluated = D->points;
    out->busy_seconds = 0;
    if (!D->lat.empty()) {
      std::vector<double> v = D->lat;
      std::sort(v.begin(), v.end());
      auto pct = [&](double q) {
        const size_t r = (size_t)std::ceil(q * (double)v.size());
        return v[std::min(v.size(), std::max<size_t>(r, 1)) - 1];
      };
      out->p50_latency_s = pct(0.50);
      out->p99_latency_s = pct(0.99);
      out->max_latency_s = v.back();
    }
    return GB_OK;
  }

  int dloop_reset_stats(gb_ctx *ctx)
  {
    DLoopState *D = ctx->dloop;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    D->submitted = D->completed = D->rejected = D->points = 0;
    D->launches = D->launched ? 1 : 0;
    D->lat.clear();
    return GB_OK;
  }

  int dloop_info(gb_ctx *ctx, long long *launches, int *idle_exits, int *running)
  {
    DLoopState *D = ctx->dloop;
    std::lock_guard<std::recursive_mutex> lk(ctx->mu);
    const bool run = loop_running(D);
    int exits = 0;
    // the device counter, read on the copy stream (the loop may be running: a relaxed read)
    DLShared sh{};
    cudaError_t e = cudaMemcpyAsync(&sh, D->d_shared, sizeof(DLShared), cudaMemcpyDeviceToHost, D->copy_stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(D->copy_stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "gb_serve_device_info");
    exits = sh.idle_exits;
    if (launches) *launches = D->launches;
    if (idle_exits) *idle_exits = exits;
    if (running) *running = run ? 1 : 0;
    return GB_OK;
  }
} // namespace gbint
