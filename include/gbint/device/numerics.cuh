// numerics.cuh -- device arithmetic shared by every gbint kernel (header-only, sm_103a).
//
// FP32-compensated evaluation rests on three rules:
//  * every constant that enters a sum (node, weight, table-axis scale) is carried as a
//    double-float pair (hi + lo, ~48-bit mantissa), so rounding a constant never becomes a
//    systematic error shared by many quadrature points;
//  * per-point arithmetic is plain FP32; its rounding errors are independent from point to
//    point and average out over the quadrature;
//  * partial sums are compensated (Kahan) in FP32 and promoted to FP64 before weights that
//    are shared by many points are applied.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

#ifndef GBINT_HD
#define GBINT_HD __host__ __device__ __forceinline__
#endif

namespace gbint
{
  namespace dev
  {
    // ---------------------------------------------------------------- double-float (hi, lo)
    struct df {
      float hi, lo;
    };

    GBINT_HD df df_from(double v)
    {
      const float h = (float)v;
      return df{h, (float)(v - (double)h)};
    }
    GBINT_HD double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

    __device__ __forceinline__ df two_sum(float a, float b)
    {
      const float s = __fadd_rn(a, b);
      const float bb = __fsub_rn(s, a);
      const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
      return df{s, e};
    }
    __device__ __forceinline__ df fast_two_sum(float a, float b)  // requires |a| >= |b|
    {
      const float s = __fadd_rn(a, b);
      return df{s, __fsub_rn(b, __fsub_rn(s, a))};
    }
    __device__ __forceinline__ df two_prod(float a, float b)
    {
      const float p = __fmul_rn(a, b);
      return df{p, __fmaf_rn(a, b, -p)};
    }
    __device__ __forceinline__ df df_add(df a, df b)
    {
      const df s = two_sum(a.hi, b.hi);
      return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
    }
    __device__ __forceinline__ df df_mul(df a, df b)
    {
      const df p = two_prod(a.hi, b.hi);
      const float e = __fadd_rn(p.lo, __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi)));
      return fast_two_sum(p.hi, e);
    }
    // a + b*c, all double-float, result double-float
    __device__ __forceinline__ df df_fma(df a, df b, df c) { return df_add(a, df_mul(b, c)); }
    __device__ __forceinline__ float df_round(df a) { return __fadd_rn(a.hi, a.lo); }

    // ---------------------------------------------------------------- compensated sum
    // Kahan summation; value() = s - c.  Written with explicit-rounding intrinsics so that
    // no contraction or reassociation can remove the compensation.
    struct Kahan {
      float s = 0.f, c = 0.f;
      __device__ __forceinline__ void add(float x)
      {
        const float y = __fsub_rn(x, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
      }
      __device__ __forceinline__ double value() const { return (double)s - (double)c; }
    };

    // ---------------------------------------------------------------- regulator (b = 1, k = 1)
    // R(x) = x/expm1(x), Rdot(x) = 2 x^2 e^x / expm1(x)^2
    // (BosonicRegulator<b=1>::RB / RBdot, DiFfRG/include/DiFfRG/physics/regulators.hh:76-99)
    __device__ __forceinline__ float reg_R(float x)
    {
      if (x < 1e-30f) return 1.f;
      return __fdiv_rn(x, expm1f(x));
    }
    GBINT_HD double reg_R(double x)
    {
      if (x == 0.0) return 1.0;
      return x / expm1(x);
    }
    GBINT_HD double reg_Rdot(double x)
    {
      if (x == 0.0) return 2.0;
      if (x > 700.0) return 0.0;
      const double em = expm1(x);
      return 2.0 * x * x * exp(x) / (em * em);
    }

    // ---------------------------------------------------------------- tables
    // Axis of a table: grid index u = scale * g(v) + shift with g = log2 (log axis) or identity;
    // scale/shift are double-float so that the index carries no systematic rounding.
    struct AxisDev {
      df scale, shift;
      int n;    // number of grid points
      int log;  // 1: log-spaced
      double scale64, shift64;
    };

    // FP32 index and fraction; u clamped to [0, n-1], cell i in [0, n-2]
    __device__ __forceinline__ float axis_frac(const AxisDev &a, float v, int &i)
    {
      const float g = a.log ? log2f(v) : v;
      // u = scale*g + shift in double-float, rounded once
      const df sg = two_prod(a.scale.hi, g);
      const float lo = __fadd_rn(__fmaf_rn(a.scale.lo, g, sg.lo), a.shift.lo);
      const df s = two_sum(sg.hi, a.shift.hi);
      float u = __fadd_rn(s.hi, __fadd_rn(s.lo, lo));
      u = fminf(fmaxf(u, 0.f), (float)(a.n - 1));  // fmaxf maps NaN to 0
      int ii = (int)u;
      ii = min(ii, a.n - 2);
      i = ii;
      return __fsub_rn(u, (float)ii);
    }
    GBINT_HD double axis_frac64(const AxisDev &a, double v, int &i)
    {
      const double g = a.log ? log2(v) : v;
      double u = a.scale64 * g + a.shift64;
      if (!(u > 0)) u = 0;
      if (u > a.n - 1) u = a.n - 1;
      int ii = (int)u;
      if (ii > a.n - 2) ii = a.n - 2;
      i = ii;
      return u - ii;
    }

    __device__ __forceinline__ float lerp32(float y0, float y1, float f) { return __fmaf_rn(f, __fsub_rn(y1, y0), y0); }
    GBINT_HD double lerp64(double y0, double y1, double f) { return y0 + f * (y1 - y0); }
  } // namespace dev
} // namespace gbint
