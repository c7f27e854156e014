// device_common.cuh -- TMA bulk staging, bounded mbarrier waits, FP64 block reductions and the
// deterministic per-integral finish shared by all gbint kernels.
#pragma once

#include <cstdint>

#include "engine_types.hh"

namespace gbint
{
  namespace dev
  {
    // error bits written to RunParams::err
    enum : int { ERR_MBAR_TIMEOUT = kErrMbarTimeout, ERR_BAD_INDEX = kErrBadIndex };

    __device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

    __device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
    {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    }
    __device__ __forceinline__ void mbar_fence_init()
    {
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
    {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                   : "memory");
    }
    // Non-tensor TMA: global -> shared bulk copy completing on an mbarrier.
    // dst/src 16-byte aligned, bytes a multiple of 16 (checked by the caller).
    __device__ __forceinline__ void tma_bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
    {
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       smem_u32(dst)),
                   "l"(src), "r"(bytes), "r"(smem_u32(bar))
                   : "memory");
    }
    __device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
    {
      uint32_t ok;
      asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
                   : "=r"(ok)
                   : "r"(smem_u32(bar)), "r"(parity)
                   : "memory");
      return ok != 0;
    }
    // Bounded wait: gives up after ~2^31 SM cycles (about a second), records ERR_MBAR_TIMEOUT
    // and returns false; callers then skip the unit so that the kernel always terminates.
    __device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, int *err,
                                                      long long limit = (1ll << 31))
    {
      const long long t0 = clock64();
      while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) {
          atomicOr(err, ERR_MBAR_TIMEOUT);
          return false;
        }
      }
      return true;
    }

    // ------------------------------------------------------------------ FP64 block reduction
    __device__ __forceinline__ double warp_sum(double v)
    {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      return v;
    }
    // deterministic for a fixed blockDim; result valid in thread 0; red has >= 32 doubles
    __device__ __forceinline__ double block_sum(double v, double *red)
    {
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      v = warp_sum(v);
      if (lane == 0) red[wid] = v;
      __syncthreads();
      const int nw = (blockDim.x + 31) >> 5;
      double r = 0.0;
      if (wid == 0) {
        r = lane < nw ? red[lane] : 0.0;
        r = warp_sum(r);
      }
      __syncthreads();
      return r;
    }

    // ------------------------------------------------------------------ per-integral finish
    // Each unit stores its FP64 partial in its slot (its position in item order, whatever order
    // the units were claimed in); the last unit of an item to arrive (atomic counter) sums the
    // item's partials in slot order with the whole block -> deterministic result, identical
    // whether the item ran alone or inside a larger batch, and whatever the unit order.
    __device__ __forceinline__ void unit_finish(const RunParams &P, int slot, int item_idx, double block_total,
                                                double *red, int *s_flag)
    {
      const ItemDev &it = P.items[item_idx];
      if (threadIdx.x == 0) {
        P.partials[slot] = block_total;
        __threadfence();
        const int prev = atomicAdd(&P.item_count[item_idx], 1);
        *s_flag = (prev == it.n_units - 1);
      }
      __syncthreads();
      if (*s_flag) {
        __threadfence();
        double v = 0.0;
        for (int u = threadIdx.x; u < it.n_units; u += blockDim.x) v += __ldcg(&P.partials[it.unit_begin + u]);
        // fixed-order tree over threads
        v = block_sum(v, red);
        if (threadIdx.x == 0) {
          P.out[item_idx] = it.args[0] + v;
          P.item_count[item_idx] = 0;
        }
      }
      __syncthreads();
    }
  } // namespace dev
} // namespace gbint
