// autotune.cc -- CTA-width autotuner of the FP32-compensated kernels.
//
// The S kinds map one quadrature row to one thread and one CTA to one work unit, so the CTA
// width fixes both the unit size (scheduling granularity of the persistent grid) and the
// occupancy.  gb_autotune times every width the kernels are built for (128, 256, 512) on the
// caller's integrals, kind by kind, and keeps the fastest in the context; batches created
// afterwards use it.  Choices are cached per GPU model in a text file (one line per kind slot:
// "<gpu name>|<SM count>|<slot>|<threads>|<ms>", slot = base kind + 8 for the double-float form),
// so that a later process on the same model skips the timing.
#include "engine.hh"
#include "kernels.hh"
#include "trace.hh"

#include <algorithm>
#include <cstdio>
#include <fstream>
#include <sstream>

namespace gbint
{
  namespace
  {
    constexpr int kCandidates[3] = {128, 256, 512};

    std::string gpu_key(gb_ctx *ctx)
    {
      cudaDeviceProp p{};
      cudaGetDeviceProperties(&p, ctx->device);
      std::string name = p.name;
      std::replace(name.begin(), name.end(), '|', '/');
      return name + "|" + std::to_string(ctx->num_sms);
    }

    // cache lines "<gpu>|<sms>|<slot>|<threads>|<ms>" -> slot -> threads
    std::map<int, int> read_cache(const char *path, const std::string &gpu)
    {
      std::map<int, int> m;
      if (!path) return m;
      std::ifstream f(path);
      std::string line;
      while (std::getline(f, line)) {
        std::vector<std::string> tok;
        std::stringstream ss(line);
        std::string t;
        while (std::getline(ss, t, '|')) tok.push_back(t);
        if (tok.size() < 4 || tok[0] + "|" + tok[1] != gpu) continue;
        const int slot = std::atoi(tok[2].c_str()), th = std::atoi(tok[3].c_str());
        if (slot >= 0 && slot < 16 && std::find(std::begin(kCandidates), std::end(kCandidates), th) != std::end(kCandidates))
          m[slot] = th;
      }
      return m;
    }

    void write_cache(const char *path, const std::string &gpu, const std::map<int, std::pair<int, double>> &best)
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
      for (const auto &kv : best) f << gpu << "|" << kv.first << "|" << kv.second.first << "|" << kv.second.second << "\n";
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
  const std::map<int, int> cached = (flags & GB_TUNE_REFRESH) ? std::map<int, int>{} : read_cache(cache_path, gpu);
  std::map<int, std::pair<int, double>> best;
  for (int kind : kinds) {
    const int slot = slot_of(kind);
    auto c = cached.find(slot);
    if (c != cached.end()) {
      ctx->threads_override[slot] = c->second;
      continue;
    }
    double best_ms = 1e300;
    int best_t = kind_default_threads(kind);
    for (int th : kCandidates) {
      ctx->threads_override[slot] = th;
      gb_batch *b = nullptr;
      int rc = build_batch(ctx, items, n, tables, n_tables, precision, &b);
      if (rc == GB_EINVAL) continue;  // this width cannot launch with these tables/records
      if (rc) {
        ctx->threads_override[slot] = 0;
        return rc;
      }
      double ms = 0;
      rc = time_batch(ctx, b, 9, ms, flush, flush_bytes);
      cudaStreamSynchronize(ctx->stream);
      free_batch(ctx, b);
      if (rc) {
        ctx->threads_override[slot] = 0;
        return rc;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best_t = th;
      }
    }
    ctx->threads_override[slot] = best_t;
    best[slot] = {best_t, best_ms};
    if (log_enabled()) log_event("autotune", jfields("\"slot\": %d, \"threads\": %d, \"ms\": %.4f", slot, best_t, best_ms));
  }
  if (!best.empty()) write_cache(cache_path, gpu, best);
  if (chosen)
    for (int k = 0; k < 16; ++k) chosen[k] = ctx->threads_override[k];
  return GB_OK;
}

extern "C" int gb_tune_set(gb_ctx *ctx, int kind_slot, int threads)
{
  if (!ctx || kind_slot < 0 || kind_slot >= 16) return GB_EINVAL;
  if (threads != 0 && std::find(std::begin(kCandidates), std::end(kCandidates), threads) == std::end(kCandidates))
    return set_error(ctx, GB_EINVAL, "gb_tune_set: threads must be 0 (default), 128, 256 or 512");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  ctx->threads_override[kind_slot] = threads;
  return GB_OK;
}
