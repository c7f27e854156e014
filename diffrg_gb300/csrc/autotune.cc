// autotune.cc -- work-unit schedule autotuner of the FP32-compensated kernels.
//
// The S kinds map quadrature rows to threads and CTAs to work units that a persistent grid
// claims from an atomic counter.  A schedule (gb_schedule) fixes the CTA width, the rows per
// thread of a unit (together: the unit size, i.e. the scheduling granularity, and the
// occupancy), the split of each row's inner loop over several threads (S3, S5Z: more threads
// per row for integrals with few rows and long inner loops), and the order the units go out in
// (item order, or largest cost first against the tail of uneven batches).  gb_autotune times
// the parameters one at a time on the caller's integrals, kind by kind, each at the best of the
// ones before, keeps the fastest in the context and records every measurement for
// gb_tune_report.  Choices are cached per GPU model in a text file (one line per kind slot:
// "<gpu name>|<SM count>|<slot>|<threads>|<ms>|<rows per thread>|<split>|<order>", slot = base
// kind + 8 for the double-float form), so that a later process on the same model skips the
// timing.
#include "engine.hh"
#include "kernels.hh"
#include "trace.hh"

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <tuple>

namespace gbint
{
  namespace
  {
    constexpr int kCandidates[3] = {128, 256, 512};
    constexpr int kRowsPerThread[3] = {1, 2, 4};
    constexpr int kSplits[3] = {1, 2, 4};
    // a candidate replaces the incumbent only when it is faster by more than this fraction
    constexpr double kMargin = 0.01;

    template <size_t N> bool one_of(int v, const int (&set)[N])
    {
      return std::find(std::begin(set), std::end(set), v) != std::end(set);
    }

    std::string gpu_key(gb_ctx *ctx)
    {
      cudaDeviceProp p{};
      cudaGetDeviceProperties(&p, ctx->device);
      std::string name = p.name;
      std::replace(name.begin(), name.end(), '|', '/');
      return name + "|" + std::to_string(ctx->num_sms);
    }

    // cache lines "<gpu>|<sms>|<slot>|<threads>|<ms>[|<rows per thread>|<split>|<order>]"
    std::map<int, gb_schedule> read_cache(const char *path, const std::string &gpu)
    {
      std::map<int, gb_schedule> m;
      if (!path) return m;
      std::ifstream f(path);
      std::string line;
      while (std::getline(f, line)) {
        std::vector<std::string> tok;
        std::stringstream ss(line);
        std::string t;
        while (std::getline(ss, t, '|')) tok.push_back(t);
        if (tok.size() < 4 || tok[0] + "|" + tok[1] != gpu) continue;
        gb_schedule sc{};
        const int slot = std::atoi(tok[2].c_str());
        sc.threads = std::atoi(tok[3].c_str());
        sc.rows_per_thread = tok.size() > 5 ? std::atoi(tok[5].c_str()) : 1;
        sc.inner_split = tok.size() > 6 ? std::atoi(tok[6].c_str()) : 1;
        sc.unit_order = tok.size() > 7 ? std::atoi(tok[7].c_str()) : GB_ORDER_ITEM;
        if (slot >= 0 && slot < 16 && one_of(sc.threads, kCandidates) && one_of(sc.rows_per_thread, kRowsPerThread) &&
            one_of(sc.inner_split, kSplits) && (sc.unit_order == GB_ORDER_ITEM || sc.unit_order == GB_ORDER_COST))
          m[slot] = sc;
      }
      return m;
    }

    void write_cache(const char *path, const std::string &gpu, const std::map<int, std::pair<gb_schedule, double>> &best)
    {
      if (!path) return;
      std::vector<std::string> keep;
      {
        std::ifstream f(path);
        std::string line;
        while (std::getline(f, line)) {
          bool replaced = false;
          for (const auto &kv : best)
            if (line.rfind(gpu + "|" + std::to_string(kv.first) + "|", 0) == 0) replaced = true;
          if (!replaced && !line.empty()) keep.push_back(line);
        }
      }
      std::ofstream f(path, std::ios::trunc);
      for (const auto &l : keep) f << l << "\n";
      for (const auto &kv : best) {
        const gb_schedule &sc = kv.second.first;
        f << gpu << "|" << kv.first << "|" << sc.threads << "|" << kv.second.second << "|" << sc.rows_per_thread << "|"
          << sc.inner_split << "|" << sc.unit_order << "\n";
      }
    }

    std::string sched_json(const gb_schedule &s)
    {
      char b[160];
      std::snprintf(b, sizeof b, "{\"threads\": %d, \"rows_per_thread\": %d, \"inner_split\": %d, \"unit_order\": \"%s\"}",
                    s.threads, s.rows_per_thread, s.inner_split, s.unit_order == GB_ORDER_COST ? "cost" : "item");
      return b;
    }

    int slot_of(int kind) { return kind_base(kind) + (kind_acc(kind) ? 8 : 0); }

    // median time (ms) of `reps` runs of the batch on the context stream; with a flush buffer
    // (larger than L2) written before each run, the runs start from a cold L2 as they do between
    // the right-hand-side evaluations of a time stepper
    int time_batch(gb_ctx *ctx, gb_batch *b, int reps, double &ms, void *flush = nullptr, size_t flush_bytes = 0)
    {
      cudaEvent_t e0, e1;
      GB_CUDA(cudaEventCreate(&e0));
      GB_CUDA(cudaEventCreate(&e1));
      std::vector<float> t;
      int rc = run_batch(ctx, b, nullptr, ctx->stream);  // warm-up
      for (int r = 0; r < reps && rc == GB_OK; ++r) {
        if (flush) cudaMemsetAsync(flush, r & 0xff, flush_bytes, ctx->stream);
        cudaEventRecord(e0, ctx->stream);
        rc = run_batch(ctx, b, nullptr, ctx->stream);
        cudaEventRecord(e1, ctx->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = set_error(ctx, GB_ECUDA, "autotune timing");
        float x = 0;
        cudaEventElapsedTime(&x, e0, e1);
        t.push_back(x);
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      if (rc) return rc;
      std::sort(t.begin(), t.end());
      ms = t[t.size() / 2];
      return GB_OK;
    }
  } // namespace
} // namespace gbint

using namespace gbint;

extern "C" int gb_autotune(gb_ctx *ctx, const gb_integral *items, int n, gb_table *const *tables, int n_tables,
                           int precision, const char *cache_path, int flags, int *chosen)
{
  if (!ctx || !items || n <= 0) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  GB_CUDA(cudaSetDevice(ctx->device));
  // kinds present in these integrals
  std::vector<int> kinds;
  {
    std::vector<gb_table *const *> tl(n, tables);
    std::vector<int> tn(n, n_tables);
    gb_batch probe;
    int rc = plan_batch(ctx, items, n, tl.data(), tn.data(), precision, &probe);
    release_axes(ctx, probe.held);
    if (rc) return rc;
    for (const auto &r : probe.runs)
      if (r.kind != K_GENERIC) kinds.push_back(r.kind);
  }
  const std::string gpu = gpu_key(ctx);
  // L2 flush buffer (twice the L2 size) when the HBM budget allows it
  void *flush = nullptr;
  size_t flush_bytes = 0;
  {
    int l2 = 0;
    if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, ctx->device) == cudaSuccess && l2 > 0) {
      flush_bytes = 2 * (size_t)l2;
      if (ctx->in_use + flush_bytes > ctx->budget || cudaMalloc(&flush, flush_bytes) != cudaSuccess) {
        cudaGetLastError();
        flush = nullptr;
      }
    }
  }
  struct FreeFlush {
    void *p;
    ~FreeFlush()
    {
      if (p) cudaFree(p);
    }
  } free_flush{flush};
  const std::map<int, gb_schedule> cached =
      (flags & GB_TUNE_REFRESH) ? std::map<int, gb_schedule>{} : read_cache(cache_path, gpu);
  std::map<int, std::pair<gb_schedule, double>> best;
  std::string report = "{\"gpu\": \"" + gpu + "\", \"kinds\": [";
  bool first_kind = true;
  for (int kind : kinds) {
    const int slot = kind_base(kind) + (kind_acc(kind) ? 8 : 0);
    const gb_schedule saved = ctx->sched[slot];
    auto c = cached.find(slot);
    if (c != cached.end()) {
      ctx->sched[slot] = c->second;
      report += std::string(first_kind ? "" : ", ") + "{\"slot\": " + std::to_string(slot) +
                ", \"cached\": true, \"chosen\": " + sched_json(resolve_schedule(ctx, kind)) + "}";
      first_kind = false;
      continue;
    }
    // median ms of one schedule (memoised); < 0 when the schedule cannot launch these integrals
    std::map<std::tuple<int, int, int, int>, double> seen;
    int rc = GB_OK;
    auto time_of = [&](gb_schedule sc) -> double {
      ctx->sched[slot] = sc;
      const gb_schedule r = resolve_schedule(ctx, kind);
      const auto key = std::make_tuple(r.threads, r.rows_per_thread, r.inner_split, r.unit_order);
      auto it = seen.find(key);
      if (it != seen.end()) return it->second;
      gb_batch *b = nullptr;
      double ms = -1;
      const int brc = build_batch(ctx, items, n, tables, n_tables, precision, &b);
      if (brc == GB_OK) {
        const int trc = time_batch(ctx, b, 9, ms, flush, flush_bytes);
        cudaStreamSynchronize(ctx->stream);
        free_batch(ctx, b);
        if (trc) {
          rc = trc;
          ms = -1;
        }
      } else if (brc != GB_EINVAL) {  // GB_EINVAL: this shape cannot launch with these tables/records
        rc = brc;
      }
      seen[key] = ms;
      return ms;
    };
    const gb_schedule def = kind_default_schedule(kind);
    const double def_ms = time_of(def);
    gb_schedule cur = def;
    double cur_ms = def_ms;
    std::string steps;
    // one parameter at a time, each at the best of the previous ones
    auto sweep = [&](const char *name, const int *vals, int nv, int gb_schedule::*field) {
      std::string row = std::string("\"") + name + "\": [";
      gb_schedule keep = cur;
      for (int v = 0; v < nv && rc == GB_OK; ++v) {
        gb_schedule sc = cur;
        sc.*field = vals[v];
        const double ms = time_of(sc);
        char e[64];
        std::snprintf(e, sizeof e, "%s[%d, %.4f]", v ? ", " : "", vals[v], ms);
        row += e;
        if (ms > 0 && (cur_ms <= 0 || ms < cur_ms * (1.0 - kMargin))) {
          keep = sc;
          cur_ms = ms;
        }
      }
      cur = keep;
      steps += (steps.empty() ? "" : ", ") + row + "]";
    };
    sweep("threads", kCandidates, 3, &gb_schedule::threads);
    sweep("rows_per_thread", kRowsPerThread, 3, &gb_schedule::rows_per_thread);
    const int kb = kind_base(kind);
    if (kb == K_S3 || kb == K_S3R || kb == K_S5Z) sweep("inner_split", kSplits, 3, &gb_schedule::inner_split);
    static const int kOrders[2] = {GB_ORDER_ITEM, GB_ORDER_COST};
    sweep("unit_order", kOrders, 2, &gb_schedule::unit_order);
    if (rc) {
      ctx->sched[slot] = saved;
      return rc;
    }
    if (cur_ms <= 0) cur = def;
    ctx->sched[slot] = cur;
    best[slot] = {cur, cur_ms};
    char tail[160];
    std::snprintf(tail, sizeof tail, ", \"default_ms\": %.4f, \"chosen_ms\": %.4f}", def_ms, cur_ms);
    report += std::string(first_kind ? "" : ", ") + "{\"slot\": " + std::to_string(slot) +
              ", \"cached\": false, \"default\": " + sched_json(def) + ", \"chosen\": " + sched_json(cur) +
              ", \"steps\": {" + steps + "}" + tail;
    first_kind = false;
    if (log_enabled())
      log_event("autotune", jfields("\"slot\": %d, \"threads\": %d, \"rows_per_thread\": %d, \"inner_split\": %d, "
                                    "\"unit_order\": %d, \"ms\": %.4f, \"default_ms\": %.4f",
                                    slot, cur.threads, cur.rows_per_thread, cur.inner_split, cur.unit_order, cur_ms,
                                    def_ms));
  }
  report += "]}";
  ctx->tune_report = report;
  if (!best.empty()) write_cache(cache_path, gpu, best);
  if (chosen)
    for (int k = 0; k < 16; ++k) chosen[k] = ctx->sched[k].threads;
  return GB_OK;
}

extern "C" int gb_tune_set(gb_ctx *ctx, int kind_slot, int threads)
{
  if (!ctx || kind_slot < 0 || kind_slot >= 16) return GB_EINVAL;
  if (threads != 0 && !one_of(threads, kCandidates))
    return set_error(ctx, GB_EINVAL, "gb_tune_set: threads must be 0 (default), 128, 256 or 512");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  ctx->sched[kind_slot].threads = threads;
  return GB_OK;
}

extern "C" int gb_tune_set_schedule(gb_ctx *ctx, int kind_slot, const gb_schedule *s)
{
  if (!ctx || !s || kind_slot < 0 || kind_slot >= 16) return GB_EINVAL;
  if ((s->threads && !one_of(s->threads, kCandidates)) || (s->rows_per_thread && !one_of(s->rows_per_thread, kRowsPerThread)) ||
      (s->inner_split && !one_of(s->inner_split, kSplits)) || (s->unit_order != GB_ORDER_ITEM && s->unit_order != GB_ORDER_COST))
    return set_error(ctx, GB_EINVAL,
                     "gb_tune_set_schedule: threads 0/128/256/512, rows_per_thread 0/1/2/4, inner_split 0/1/2/4, "
                     "unit_order GB_ORDER_ITEM/GB_ORDER_COST");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  ctx->sched[kind_slot] = *s;
  return GB_OK;
}

extern "C" int gb_tune_get_schedule(gb_ctx *ctx, int kind_slot, gb_schedule *out)
{
  if (!ctx || !out || kind_slot < 0 || kind_slot >= 16) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  const int kind = (kind_slot & 7) | ((kind_slot & 8) ? K_ACC : 0);
  *out = resolve_schedule(ctx, kind);
  return GB_OK;
}

extern "C" int gb_tune_report(gb_ctx *ctx, char *buf, size_t cap, size_t *len)
{
  if (!ctx) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  const std::string &r = ctx->tune_report.empty() ? std::string("{}") : ctx->tune_report;
  if (len) *len = r.size();
  if (buf && cap) {
    const size_t m = std::min(cap - 1, r.size());
    std::memcpy(buf, r.data(), m);
    buf[m] = 0;
  }
  return GB_OK;
}
