// user_batch.cuh -- the fused kernel of the C++ class templates: any number of integrals of one
// user KERNEL (one family, one argument signature) in one persistent launch.
//
// Work units are (integral, 32 x 1..8 grid points, see ppt_for): one warp's.  CTAs are two
// warps, and every warp takes units from an atomic counter on its own, so a batch of small
// integrals spreads over the SMs in steps of two warps rather than of whole eight-warp CTAs.
// Before its first unit a CTA stages the arrays every integral of the launch
// reads -- the quadrature nodes and weights of each axis, the Matsubara rule, and the data of
// the interpolator arguments (TexLinearInterpolator*, LinearInterpolator*) -- into shared memory
// with non-tensor TMA bulk copies (cp.async.bulk ... mbarrier::complete_tx::bytes) and waits on
// an mbarrier with a bounded spin; an integral whose arrays are the staged ones reads them from
// shared memory, any other reads global memory.  A wait that runs out records an error bit and
// the CTA keeps reading global memory (results stay correct).  Points are evaluated in NT
// (FAM::eval, the reference's maps and Jacobians), reduced per unit in FP64 (float results:
// Kahan-compensated FP32 per thread first), and the last unit of an integral to arrive sums the
// integral's unit partials in unit order -- so a result is bit-identical whether its integral ran
// alone or in a batch of any size.
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>

#include <cuda_runtime.h>

#include "gbint/device/families.cuh"

namespace gbint
{
  namespace ub
  {
    constexpr int kThreads = 64;          // CTA size: two warps, each an independent worker
#ifndef GBINT_UB_MIN_CTAS
#define GBINT_UB_MIN_CTAS 8
#endif
    // resident CTAs per SM the register allocation is held to: 8 (16 warps, <= 128 registers
    // a thread) keeps the FP64 pipe of GB300 busy for the generated KERNELs; a translation
    // unit whose KERNEL spills heavily at 128 may define GBINT_UB_MIN_CTAS 6 (<= 168) first
    constexpr int kMinCtas = GBINT_UB_MIN_CTAS;
    constexpr int kUnitLanes = 32;        // a work unit is one warp's
    constexpr int kMaxStage = 24;         // staged arrays per launch
    constexpr unsigned kStageAlign = 16;  // TMA bulk copies: 16-byte addresses and sizes
    enum : int { ERR_STAGE_TIMEOUT = 1, ERR_STAGE_ALIGN = 2 };

    // Points per lane of an integral's work units, from the integral's own size only -- so its
    // unit decomposition, and with it the rounding of its result, is the same alone and in any
    // batch.  A unit is one warp's (32 x ppt points): the reference examples' 512-point angle
    // grids give 16 units each, which the warps of the whole GPU pull one at a time, so no SM
    // ends up with a whole extra CTA's share; larger integrals take 2, 4 and 8 points per lane,
    // which keeps the per-unit work (claim, descriptor, reduction) small against the points.
    __host__ __device__ constexpr int ppt_for(long long n_points)
    {
      return n_points <= 1024 ? 1 : (n_points <= 8192 ? 2 : (n_points <= 65536 ? 4 : 8));
    }
    __host__ __device__ constexpr long long unit_points(long long n_points)
    {
      return (long long)kUnitLanes * ppt_for(n_points);
    }

    // ------------------------------------------------------------------ argument packs
    // A trivially copyable tuple of the KERNEL's extra arguments (kernel parameters and batch
    // items are copied bytewise to the device).
    template <class... T> struct ArgPack;
    template <> struct ArgPack<> {
    };
    template <class H, class... R> struct ArgPack<H, R...> {
      H h;
      ArgPack<R...> r;
    };
    inline ArgPack<> make_pack() { return {}; }
    template <class H, class... R> ArgPack<H, R...> make_pack(const H &h, const R &...r)
    {
      return ArgPack<H, R...>{h, make_pack(r...)};
    }
    template <int I, class H, class... R> __host__ __device__ __forceinline__ auto &pget(ArgPack<H, R...> &p)
    {
      if constexpr (I == 0)
        return p.h;
      else
        return pget<I - 1>(p.r);
    }
    template <int I, class H, class... R>
    __host__ __device__ __forceinline__ const auto &pget(const ArgPack<H, R...> &p)
    {
      if constexpr (I == 0)
        return p.h;
      else
        return pget<I - 1>(p.r);
    }

    // ------------------------------------------------------------------ staging plan
    // Arrays copied to shared memory at CTA start: src (global, 16-byte aligned), off (shared
    // offset), bytes (a multiple of 16 that stays inside the source allocation: the library
    // pads the device rule arrays and interpolator buffers to 16 bytes).
    struct StagePlan {
      int n = 0;
      unsigned total = 0;
      const void *src[kMaxStage] = {};
      unsigned off[kMaxStage] = {};
      unsigned bytes[kMaxStage] = {};
    };
    // one batch entry: the integral's maps/rules and its KERNEL arguments
    template <typename ctype, class... T> struct Item {
      gbint::fam::Params<ctype> P;
      ArgPack<T...> args;
    };

    // The fields of a batch's entries that differ between its integrals -- bit 0 the maps and
    // rules (Params), bit 1 + I KERNEL argument I.  Integral i's varying fields sit at
    // rows + i * stride + off[field] (16-byte aligned); every other field is item 0's, which the
    // kernel receives by value.  A grid of requests usually varies in one or two scalars (the
    // external momentum), so a batch uploads a few bytes per integral instead of its whole
    // entry (~1 KB with interpolator arguments).
    constexpr int kMaxFields = 25;
    struct Varying {
      unsigned mask = 0;
      unsigned stride = 0;
      unsigned short off[kMaxFields] = {};
    };
    // host: call f(field, address, bytes) for the Params and every argument of an entry
    template <typename ctype, class... T, class F, size_t... I>
    void for_each_field(const Item<ctype, T...> &it, F &&f, std::index_sequence<I...>)
    {
      f(0, static_cast<const void *>(&it.P), sizeof(it.P));
      (f((int)I + 1, static_cast<const void *>(&pget<(int)I>(it.args)), sizeof(pget<(int)I>(it.args))), ...);
    }

    // interpolator arguments with device tables opt in with a member type gbint_stageable_table
    // and device_data(), table_bytes(), retarget(const void *) -- see gbint/interpolators.hh
    template <class A, class = void> struct is_stageable : std::false_type {
    };
    template <class A> struct is_stageable<A, std::void_t<typename A::gbint_stageable_table>> : std::true_type {
    };

#ifdef __CUDACC__
    __device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
    __device__ __forceinline__ void bar_init(uint64_t *bar)
    {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(saddr(bar)) : "memory");
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __device__ __forceinline__ void bar_expect(uint64_t *bar, uint32_t bytes)
    {
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
    }
    __device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
    {
      asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                       saddr(dst)),
                   "l"(src), "r"(bytes), "r"(saddr(bar))
                   : "memory");
    }
    __device__ __forceinline__ bool bar_try(uint64_t *bar, uint32_t parity)
    {
      uint32_t ok;
      asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
                   : "=r"(ok)
                   : "r"(saddr(bar)), "r"(parity)
                   : "memory");
      return ok != 0;
    }
    // bounded wait: ~2^27 SM cycles (~65 ms at 2 GHz) for a few KB, then give up
    __device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity, long long limit = (1ll << 27))
    {
      const long long t0 = clock64();
      while (!bar_try(bar, parity))
        if (clock64() - t0 > limit) return false;
      return true;
    }

    __device__ __forceinline__ double warp_sum(double v)
    {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      return v;
    }

    // retarget the staged arrays of one integral to their shared-memory copies
    template <typename ctype>
    __device__ __forceinline__ void retarget_params(gbint::fam::Params<ctype> &P, const StagePlan &plan, const char *sm)
    {
      for (int s = 0; s < plan.n; ++s) {
        const void *src = plan.src[s];
        const ctype *dst = reinterpret_cast<const ctype *>(sm + plan.off[s]);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          if (P.x[a] == src) P.x[a] = dst;
          if (P.w[a] == src) P.w[a] = dst;
        }
        if (P.mx == src) P.mx = dst;
        if (P.mw == src) P.mw = dst;
      }
    }
    template <class A> __device__ __forceinline__ void retarget_arg(A &a, const StagePlan &plan, const char *sm)
    {
      if constexpr (is_stageable<A>::value) {
        const void *d = a.device_data();
        for (int s = 0; s < plan.n; ++s)
          if (d == plan.src[s]) a.retarget(sm + plan.off[s]);
      }
    }
    template <class... T, size_t... I>
    __device__ __forceinline__ void retarget_args(ArgPack<T...> &p, const StagePlan &plan, const char *sm,
                                                  std::index_sequence<I...>)
    {
      (retarget_arg(pget<(int)I>(p), plan, sm), ...);
    }
    // the varying arguments of one integral over item 0's
    template <int I, class... T>
    __device__ __forceinline__ void overlay_arg(ArgPack<T...> &a, const char *row, const Varying &v)
    {
      if ((v.mask >> (I + 1)) & 1u) {
        auto &dst = pget<I>(a);
        memcpy(static_cast<void *>(&dst), row + v.off[I + 1], sizeof(dst));
      }
    }
    template <class... T, size_t... I>
    __device__ __forceinline__ void overlay_args(ArgPack<T...> &a, const char *row, const Varying &v,
                                                 std::index_sequence<I...>)
    {
      (overlay_arg<(int)I>(a, row, v), ...);
    }
    template <class FAM, class KERNEL, typename NT, typename ctype, class... T, size_t... I>
    __device__ __forceinline__ NT eval_point(const gbint::fam::Params<ctype> &P, long long idx,
                                             const ArgPack<T...> &a, std::index_sequence<I...>)
    {
      return FAM::template eval<KERNEL, NT>(P, idx, pget<(int)I>(a)...);
    }

    // Persistent batched kernel.  COMP: the result type's components (C scalar components of
    // type S, get(v, c) on the device).  Integral i is item0 (by value) with its varying fields
    // read from rows (see Varying); rows == nullptr: every integral is item0.
    // unit_begin[i] .. unit_begin[i+1]: the units of integral i (unit_begin == nullptr: all of
    // item0's units).  partials: C doubles per unit; arrivals: one counter per integral (zeroed
    // before the launch and again by the finishing warp); results: C doubles per integral.
    template <class FAM, class KERNEL, typename NT, typename ctype, class COMP, class... T>
    __global__ void __launch_bounds__(kThreads, kMinCtas)
        k_user_batch(const Item<ctype, T...> item0, const char *rows, const Varying var, const int *unit_begin,
                     int units_per_item, int n_items, int n_units, const StagePlan plan, double *partials, int *unit_counter, int *arrivals,
                     double *results, int *err)
    {
      static_assert(sizeof...(T) + 1 <= kMaxFields, "integrator batch: at most 24 KERNEL arguments");
      constexpr int C = COMP::C;
      using S = typename COMP::S;
      extern __shared__ __align__(16) char stage[];
      __shared__ __align__(8) uint64_t bar;
      __shared__ int s_staged;
      const int lane = threadIdx.x & 31;

      // stage the launch's shared arrays once per CTA
      if (threadIdx.x == 0) {
        int ok = plan.n > 0 ? 1 : 0;
        for (int s = 0; s < plan.n; ++s)
          if ((reinterpret_cast<uintptr_t>(plan.src[s]) | plan.off[s] | plan.bytes[s]) & (kStageAlign - 1)) ok = 0;
        if (plan.n > 0 && !ok) atomicOr(err, ERR_STAGE_ALIGN);
        if (ok) {
          bar_init(&bar);
          bar_expect(&bar, plan.total);
          for (int s = 0; s < plan.n; ++s) bulk_g2s(stage + plan.off[s], plan.src[s], plan.bytes[s], &bar);
        }
        s_staged = ok;
      }
      __syncthreads();
      bool staged = s_staged != 0;
      if (staged) {
        staged = bar_wait(&bar, 0);
        if (!staged) atomicOr(err, ERR_STAGE_TIMEOUT);
        // the CTA decides together: any thread that gave up makes all read global memory
        staged = __syncthreads_and(staged ? 1 : 0) != 0;
      }

      // every warp pulls units on its own: claim, evaluate, reduce, and finish the integral when
      // its unit is the last to arrive
      for (;;) {
        int u = 0;
        if (lane == 0) u = atomicAdd(unit_counter, 1);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= n_units) break;
        // the unit's integral: unit_begin is sorted, binary search (uniform across the warp)
        int item = 0, first = 0, units_of = n_units;
        if (units_per_item > 0) {  // every integral has the same number of units
          item = u / units_per_item;
          first = item * units_per_item;
          units_of = units_per_item;
        } else if (unit_begin) {
          int lo = 0, hi = n_items - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&unit_begin[mid]) <= u)
              lo = mid;
            else
              hi = mid - 1;
          }
          item = lo;
          first = __ldg(&unit_begin[item]);
          units_of = __ldg(&unit_begin[item + 1]) - first;
        }
        gbint::fam::Params<ctype> P = item0.P;
        ArgPack<T...> A = item0.args;
        if (rows) {
          const char *row = rows + (size_t)item * var.stride;
          if (var.mask & 1u) memcpy(static_cast<void *>(&P), row + var.off[0], sizeof(P));
          overlay_args(A, row, var, std::index_sequence_for<T...>{});
        }
        if (staged) {
          retarget_params(P, plan, stage);
          retarget_args(A, plan, stage, std::index_sequence_for<T...>{});
        }
        const long long n_points = FAM::points(P);
        const int ppt = ppt_for(n_points);
        const long long begin = (long long)(u - first) * kUnitLanes * ppt;
        double acc[C];
        if constexpr (std::is_same_v<S, float>) {
          float s[C], c[C];  // Kahan per component
#pragma unroll
          for (int m = 0; m < C; ++m) s[m] = c[m] = 0.f;
#pragma unroll 1
          for (int k = 0; k < ppt; ++k) {
            const long long idx = begin + lane + k * kUnitLanes;
            if (idx < n_points) {
              const NT v = eval_point<FAM, KERNEL, NT>(P, idx, A, std::index_sequence_for<T...>{});
#pragma unroll
              for (int m = 0; m < C; ++m) {
                const float y = __fsub_rn((float)COMP::get(v, m), c[m]);
                const float tt = __fadd_rn(s[m], y);
                c[m] = __fsub_rn(__fsub_rn(tt, s[m]), y);
                s[m] = tt;
              }
            }
          }
#pragma unroll
          for (int m = 0; m < C; ++m) acc[m] = (double)s[m] - (double)c[m];
        } else {
#pragma unroll
          for (int m = 0; m < C; ++m) acc[m] = 0.0;
#pragma unroll 1
          for (int k = 0; k < ppt; ++k) {
            const long long idx = begin + lane + k * kUnitLanes;
            if (idx < n_points) {
              const NT v = eval_point<FAM, KERNEL, NT>(P, idx, A, std::index_sequence_for<T...>{});
#pragma unroll
              for (int m = 0; m < C; ++m) acc[m] += (double)COMP::get(v, m);
            }
          }
        }
#pragma unroll
        for (int m = 0; m < C; ++m) acc[m] = warp_sum(acc[m]);
        int last = 0;
        if (lane == 0) {
#pragma unroll
          for (int m = 0; m < C; ++m) partials[(size_t)u * C + m] = acc[m];
          __threadfence();
          last = (atomicAdd(&arrivals[item], 1) == units_of - 1);
        }
        if (__shfl_sync(0xffffffffu, last, 0)) {  // the integral's unit partials in unit order
          __threadfence();
          double v[C];
#pragma unroll
          for (int m = 0; m < C; ++m) v[m] = 0.0;
          for (int i = lane; i < units_of; i += kUnitLanes)
#pragma unroll
            for (int m = 0; m < C; ++m) v[m] += __ldcg(&partials[(size_t)(first + i) * C + m]);
#pragma unroll
          for (int m = 0; m < C; ++m) v[m] = warp_sum(v[m]);
          if (lane == 0) {
#pragma unroll
            for (int m = 0; m < C; ++m) results[(size_t)item * C + m] = v[m];
            arrivals[item] = 0;
          }
        }
      }
      // a staging wait that gave up: wait (bounded again) for the copies still in flight before
      // the CTA's shared memory is released
      if (s_staged && !staged && threadIdx.x == 0) bar_wait(&bar, 0, 1ll << 31);
    }
#endif // __CUDACC__
  } // namespace ub
} // namespace gbint
