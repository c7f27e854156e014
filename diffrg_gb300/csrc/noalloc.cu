// noalloc.cu -- gb_get_noalloc: one FP64 integral evaluated without allocating device memory.
//
// Who needs it: callers that cannot let this library call cudaMalloc or cudaFree while they
// integrate.  Two kinds are common.  (1) A host program whose device memory belongs to another
// allocator: a caching or pool allocator (a PyTorch process, an RMM pool) that reserved nearly
// all of HBM at start-up, or a code that grants each library a fixed budget once -- a cudaMalloc
// from here would fail, or would take memory the owner has already promised elsewhere.
// (2) A caller on a latency-critical path with work in flight on other streams: cudaFree waits
// for the whole device, and cudaMalloc may, so one allocating call stalls everyone's kernels.
// gb_get builds a small batch per call and allocates its scratch; this entry point keeps its
// scratch in a fixed file-scope device array instead, and otherwise computes the same integral
// with the same kernel body (dev::eval_point_fp64 and the same reduction order).
//
// Scratch: g_noalloc_scratch below, GB_NOALLOC_SCRATCH_BYTES (36 KiB) per device, resident from
// module load until process exit on every GPU that loads the library.  It holds the integral's
// descriptor, two counters, the result and one FP64 partial per work unit of 1024 grid points,
// so one call accepts at most GB_NOALLOC_MAX_POINTS = 4096 * 1024 = 4,194,304 grid points (nodes
// per axis multiplied; the +-q0 pairs of finite-T axes count once).  Larger integrals are
// rejected with GB_EINVAL and a message naming the limit; nothing is launched for them.
//
// Every call on a device shares the one array and finds the previous call's contents in it: the
// descriptor is rewritten and the two counters are cleared on the stream before each launch, and
// the result slot is written by the kernel before it is read.  Calls through one context
// serialise on the context mutex and complete (the context's stream is synchronised) before they
// return; calls through two contexts on the same device whose work overlaps on the GPU race on
// the array and must not be made.
//
// The host cannot use the array's name as a device address: in host code it names a host-side
// stand-in, and a kernel given that pointer would fault or silently use the wrong memory.  The
// first call on each device therefore resolves the address with cudaGetSymbolAddress, with that
// device current, checks the return code and caches the address per device ordinal.  That lookup
// is part of the first call's set-up: make the first call on each device before any CUDA stream
// capture begins.  New quadrature orders and axes fill host-side caches and
// are copied into the context's node pool, which was allocated once at gb_ctx_create; no device
// or pinned memory is allocated by this entry point.  The call runs eagerly and waits for the
// context's stream (it is not recorded into a graph being captured elsewhere); under CUDA's
// capture rules that wait is an unsafe call, so a global- or thread-local-mode capture open at
// the time is invalidated (tests/test_zz_no_alloc.py runs it under a relaxed-mode capture).
#include <cstddef>
#include <mutex>

#include "device_common.cuh"
#include "engine.hh"
#include "integrands.cuh"
#include "kernels.hh"

namespace gbint
{
  int prepare_item_fp64(gb_ctx *ctx, const gb_integral &g, gb_table *const *tables, int n_tables, ItemDev &it,
                        uint64_t &grid_points, std::vector<AxisKey> &hold);

  namespace
  {
    constexpr int kNoAllocMaxUnits = GB_NOALLOC_MAX_POINTS / kGenericUnitPoints;
    static_assert(GB_NOALLOC_MAX_POINTS % kGenericUnitPoints == 0, "unit size must divide the point limit");

    struct NoAllocScratch {
      ItemDev item;
      int unit_counter;
      int item_count;
      int pad[2];
      double result;
      double partials[kNoAllocMaxUnits];
    };
    static_assert(sizeof(NoAllocScratch) <= GB_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

    // the scratch: fixed size, one copy per device, lives until process exit
    static __device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES];

    std::mutex g_addr_mu;
    void *g_addr[64] = {};  // device address of g_noalloc_scratch per device ordinal

    // The generic FP64 kernel with its work units implied (unit u = grid points
    // [u*1024, (u+1)*1024)) and all scratch -- descriptor, counters, partials, result -- in the
    // static array.  Reduction order equals the generic kernel's, so results agree bitwise.
    __global__ void __launch_bounds__(kGenericThreads) k_generic_noalloc(NoAllocScratch *S, long long points,
                                                                       const double *pv, const double *pw,
                                                                       const TableDev *tabs)
    {
      __shared__ double red[32];
      __shared__ int s_unit, s_flag;
      __shared__ TableDev sT[4];
      const ItemDev &it = S->item;
      RunParams P{};
      P.items = &S->item;
      P.partials = S->partials;
      P.item_count = &S->item_count;
      P.out = &S->result;
      if (threadIdx.x < 4) {
        const int slot = it.tab[threadIdx.x];
        if (slot >= 0) sT[threadIdx.x] = tabs[slot];
      }
      for (;;) {
        if (threadIdx.x == 0) s_unit = atomicAdd(&S->unit_counter, 1);
        __syncthreads();
        const int u = s_unit;
        if (u >= it.n_units) break;
        const long long begin = (long long)u * kGenericUnitPoints;
        const long long count = min((long long)kGenericUnitPoints, points - begin);
        double acc = 0.0;
#pragma unroll 1
        for (int k = 0; k < kGenericPPT; ++k) {
          const int local = threadIdx.x + k * blockDim.x;
          if (local < count) acc += dev::eval_point_fp64(it, begin + local, pv, pw, sT);
        }
        const double tot = dev::block_sum(acc, red);
        dev::unit_finish(P, u, 0, tot, red, &s_flag);
      }
    }

    int scratch_address(gb_ctx *ctx, NoAllocScratch **out)
    {
      if (ctx->device < 0 || ctx->device >= 64) return set_error(ctx, GB_ENODEV, "device ordinal beyond 63");
      std::lock_guard<std::mutex> lk(g_addr_mu);
      if (!g_addr[ctx->device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);  // device is current
        if (e != cudaSuccess || !p) return cuda_fail(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_addr[ctx->device] = p;
      }
      *out = static_cast<NoAllocScratch *>(g_addr[ctx->device]);
      return GB_OK;
    }
  } // namespace
} // namespace gbint

using namespace gbint;

extern "C" int gb_get_noalloc(gb_ctx *ctx, const gb_integral *item, gb_table *const *tables, int n_tables,
                              double *out)
{
  if (!ctx || !item || !out) return GB_EINVAL;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  NoAllocScratch *S = nullptr;
  int rc = scratch_address(ctx, &S);
  if (rc) return rc;
  ItemDev it;
  uint64_t points = 0;
  // the axes stay held (not evictable) until the result is back; the node pool keeps its
  // pre-allocated capacity, so this holds no device memory of its own
  struct Hold {
    gb_ctx *c;
    std::vector<AxisKey> keys;
    ~Hold() { release_axes(c, keys); }
  } hold{ctx, {}};
  rc = prepare_item_fp64(ctx, *item, tables, n_tables, it, points, hold.keys);
  if (rc) return rc;
  if (points > (uint64_t)GB_NOALLOC_MAX_POINTS)
    return set_error(ctx, GB_EINVAL,
                     "gb_get_noalloc: the integral has " + std::to_string(points) +
                         " grid points; the allocation-free entry point accepts at most " +
                         std::to_string(GB_NOALLOC_MAX_POINTS) + " (use gb_get)");
  const int n_units = (int)((points + kGenericUnitPoints - 1) / kGenericUnitPoints);
  it.unit_begin = 0;
  it.n_units = n_units;
  it.rows = (int)points;
  cudaStream_t s = ctx->stream;
  // descriptor in, counters cleared (the array keeps the previous call's contents)
  e = cudaMemcpyAsync(&S->item, &it, sizeof(ItemDev), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(&S->unit_counter, 0, 2 * sizeof(int), s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gb_get_noalloc set-up copy");
  const int ctas = std::min(n_units, ctx->num_sms * 8);
  k_generic_noalloc<<<ctas, kGenericThreads, 0, s>>>(S, (long long)points, ctx->pool.d_v, ctx->pool.d_w, ctx->d_dir);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "k_generic_noalloc launch");
  e = cudaMemcpyAsync(out, &S->result, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gb_get_noalloc result copy");
  return GB_OK;
}
