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
    //
    // FP32 form built only from correctly rounded operations (add, mul, fma, div), so that its
    // rounding errors have no preferred sign, and with truncation / constant errors below 1e-10:
    //  * x < 1/4: Bernoulli series R = 1 - x/2 + x^2 (1/12 - x^2/720 + x^4/30240 - x^6/1209600);
    //  * x >= 1/4: e^x - 1 = 2^n (1 + em) - 1 with x log2(e) = n + f split in double-float,
    //    em = e^(f ln 2) - 1 from its Taylor series (|f ln 2| <= 0.35, 9 terms), then one fma and
    //    one division.  (The library expm1f was measured to carry a ~3e-9 relative bias.)
    __device__ __forceinline__ float reg_R(float x)
    {
      if (x < 0.25f) {
        if (x < 1e-30f) return 1.f;
        const float y = __fmul_rn(x, x);
        float p = __fmaf_rn(y, -8.2671957671957672e-07f, 3.3068783068783070e-05f);  // -1/1209600, 1/30240
        p = __fmaf_rn(y, p, -1.3888888888888889e-03f);                                 // -1/720
        // 1/12 as a double-float pair: h = y (1/12 + y p)
        const float c12_hi = 8.33333358e-02f, c12_lo = -2.48352705e-09f;
        const float h = __fmaf_rn(y, __fmaf_rn(y, p, c12_lo), __fmul_rn(y, c12_hi));
        // small part first, then a single rounding of 1 + s (rounding 1 - x/2 on its own is
        // always upward for x below the ulp of 1 and biases R)
        return __fadd_rn(1.0f, __fmaf_rn(-0.5f, x, h));
      }
      if (x > 88.0f) return 0.f;  // x e^-x < 1e-36
      // t = x log2(e) in double-float
      const float L2E_hi = 1.44269502e+00f, L2E_lo = 1.92596299e-08f;
      const float t_hi = __fmul_rn(x, L2E_hi);
      const float t_lo = __fmaf_rn(x, L2E_lo, __fmaf_rn(x, L2E_hi, -t_hi));
      const float n = rintf(t_hi);
      const float f = __fadd_rn(__fsub_rn(t_hi, n), t_lo);  // t_hi - n is exact
      // r = f ln2 in double-float
      const float LN2_hi = 6.93147182e-01f, LN2_lo = -1.90465421e-09f;
      const float r_hi = __fmul_rn(f, LN2_hi);
      const float r_lo = __fmaf_rn(f, LN2_lo, __fmaf_rn(f, LN2_hi, -r_hi));
      // e^r - 1 = r + r^2 (1/2 + r/6 + r^2/24 + ... + r^7/362880)
      float q = __fmaf_rn(r_hi, 2.75573192239858907e-06f, 2.48015873015873016e-05f);
      q = __fmaf_rn(r_hi, q, 1.98412698412698413e-04f);
      q = __fmaf_rn(r_hi, q, 1.38888888888888889e-03f);
      q = __fmaf_rn(r_hi, q, 8.33333333333333333e-03f);
      q = __fmaf_rn(r_hi, q, 4.16666666666666667e-02f);
      // 1/6 as a double-float pair (its FP32 rounding alone biased R by ~6e-10)
      const float c6_hi = 1.66666672e-01f, c6_lo = -4.96705388e-09f;
      q = __fmaf_rn(r_hi, q, c6_hi);
      q = __fmaf_rn(r_hi, q, 0.5f);
      const float r2 = __fmul_rn(r_hi, r_hi);
      const float em =
          __fadd_rn(r_hi, __fmaf_rn(r2, q, __fmaf_rn(__fmul_rn(r2, r_hi), c6_lo, r_lo)));
      // e^x - 1 = 2^n em + (2^n - 1), one rounding
      const float pn = ldexpf(1.0f, (int)n);
      const float D = __fmaf_rn(pn, em, __fsub_rn(pn, 1.0f));
      return __fdiv_rn(x, D);
    }
    GBINT_HD double reg_R(double x)
    {
      if (x == 0.0) return 1.0;
      return x / expm1(x);
    }

    // ---------------------------------------------------------------- double-float helpers
    __device__ __forceinline__ df df_norm(float hi, float lo) { return fast_two_sum(hi, lo); }
    __device__ __forceinline__ df df_add_f(df a, float b)
    {
      const df s = two_sum(a.hi, b);
      return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
    }
    // 1/a: one Newton step on an approximate FP32 reciprocal (the residual e = 1 - g a is
    // formed by fma; the step restores ~44 bits whatever the last bits of g)
    __device__ __forceinline__ df df_rcp(df a)
    {
      const float g = __fdividef(1.0f, a.hi);
      const float e = __fsub_rn(__fmaf_rn(-g, a.hi, 1.0f), __fmul_rn(g, a.lo));
      return fast_two_sum(g, __fmul_rn(g, e));
    }
    // y0 + f (y1 - y0) for FP32 table values, result double-float
    __device__ __forceinline__ df lerp_df(float y0, float y1, float f)
    {
      const df d = two_sum(y1, -y0);
      const df p = two_prod(f, d.hi);
      const df s = two_sum(y0, p.hi);
      return fast_two_sum(s.hi, __fadd_rn(s.lo, __fmaf_rn(f, d.lo, p.lo)));
    }
    // the same with a double-float fraction f = fh + fl
    __device__ __forceinline__ df lerp_dff(float y0, float y1, df f)
    {
      const df d = two_sum(y1, -y0);
      const df p = two_prod(f.hi, d.hi);
      const df s = two_sum(y0, p.hi);
      return fast_two_sum(s.hi, __fadd_rn(s.lo, __fmaf_rn(f.hi, d.lo, __fmaf_rn(f.lo, d.hi, p.lo))));
    }
    // sqrt of a double-float: the correctly rounded FP32 root plus one Newton correction,
    // (x - s^2) / 2s with x - s^2 formed by fma (~2^-44 relative)
    __device__ __forceinline__ df df_sqrt(df x)
    {
      if (!(x.hi > 0.f)) return df{0.f, 0.f};
      const float s = __fsqrt_rn(x.hi);
      const float e = __fadd_rn(__fmaf_rn(-s, s, x.hi), x.lo);
      return fast_two_sum(s, __fdividef(e, __fadd_rn(s, s)));
    }
    // a + f (b - a) for double-float a, b
    __device__ __forceinline__ df lerp_dd(df a, df b, float f)
    {
      const df d = df_add(b, df{-a.hi, -a.lo});
      return df_add(a, df_mul(df{f, 0.f}, d));
    }

    // R(x) = x/expm1(x) for a double-float x, double-float result with a relative error of a few
    // 1e-9 (the FP32 Taylor polynomial of e^r - 1 beyond its quadratic term is the limit).
    // EXACT_LOW: the low-order terms that carry most of the value are formed in double-float too
    // (x^2 in the series branch; r^2/2 and r^3/6 of e^r - 1 in the exponential branch), which
    // takes the regulator from ~1e-8 to ~1e-10 relative error at ~30 more instructions; used
    // where an integral rests on a few thousand points.
    template <bool EXACT_LOW = false> __device__ __forceinline__ df reg_R_df(df x)
    {
      const float xh = x.hi, xl = x.lo;
      if (xh < 0.25f) {
        if (xh < 1e-30f) return df{1.f, 0.f};
        const float y = __fmul_rn(xh, xh);
        float p = __fmaf_rn(y, -8.2671957671957672e-07f, 3.3068783068783070e-05f);
        p = __fmaf_rn(y, p, -1.3888888888888889e-03f);
        const float c12_hi = 8.33333358e-02f, c12_lo = -2.48352705e-09f;
        float h = __fmaf_rn(y, __fmaf_rn(y, p, c12_lo), __fmul_rn(y, c12_hi));
        if constexpr (EXACT_LOW) {
          // y c12 with y = x^2 exact (two_prod plus the low part of x): h = y c12 + y^2 p
          const df yy = two_prod(xh, xh);
          const float yl = __fmaf_rn(2.0f * xh, xl, yy.lo);
          const df yc = two_prod(yy.hi, c12_hi);
          h = __fadd_rn(yc.hi, __fadd_rn(yc.lo, __fmaf_rn(yl, c12_hi, __fmaf_rn(yy.hi, c12_lo, __fmul_rn(__fmul_rn(y, y), p)))));
        }
        const df s = two_sum(__fmul_rn(-0.5f, xh), h);  // -x/2 exact
        const df r = fast_two_sum(1.0f, s.hi);
        return df_norm(r.hi, __fadd_rn(r.lo, __fmaf_rn(-0.5f, xl, s.lo)));
      }
      if (xh > 88.0f) return df{0.f, 0.f};
      const float L2E_hi = 1.44269502e+00f, L2E_lo = 1.92596299e-08f;
      const float t_hi = __fmul_rn(xh, L2E_hi);
      const float t_lo =
          __fadd_rn(__fmaf_rn(xh, L2E_hi, -t_hi), __fmaf_rn(xh, L2E_lo, __fmul_rn(xl, L2E_hi)));
      const float n = rintf(t_hi);
      const float f_hi = __fsub_rn(t_hi, n);  // exact; f = f_hi + t_lo
      const float LN2_hi = 6.93147182e-01f, LN2_lo = -1.90465421e-09f;
      const float r_hi0 = __fmul_rn(f_hi, LN2_hi);
      const float r_lo0 =
          __fadd_rn(__fmaf_rn(f_hi, LN2_hi, -r_hi0), __fmaf_rn(f_hi, LN2_lo, __fmul_rn(t_lo, LN2_hi)));
      const df r = fast_two_sum(r_hi0, r_lo0);
      float q = __fmaf_rn(r.hi, 2.75573192239858907e-06f, 2.48015873015873016e-05f);
      q = __fmaf_rn(r.hi, q, 1.98412698412698413e-04f);
      q = __fmaf_rn(r.hi, q, 1.38888888888888889e-03f);
      q = __fmaf_rn(r.hi, q, 8.33333333333333333e-03f);
      q = __fmaf_rn(r.hi, q, 4.16666666666666667e-02f);
      const float c6_hi = 1.66666672e-01f, c6_lo = -4.96705388e-09f;
      q = __fmaf_rn(r.hi, q, c6_hi);
      q = __fmaf_rn(r.hi, q, 0.5f);
      // em = r + r^2 q: r^2 and r^2 q as double-float
      const df r2 = two_prod(r.hi, r.hi);
      const float r2l = __fmaf_rn(2.0f * r.hi, r.lo, r2.lo);
      df em;
      if constexpr (!EXACT_LOW) {
        const df tq = two_prod(r2.hi, q);
        const float tl = __fmaf_rn(r2l, q, __fmaf_rn(__fmul_rn(r2.hi, r.hi), c6_lo, tq.lo));
        const df e0 = two_sum(r.hi, tq.hi);
        em = fast_two_sum(e0.hi, __fadd_rn(e0.lo, __fadd_rn(r.lo, tl)));
      } else {
        // em = r + r^2/2 + r^3/6 + r^4 q4, q4 = 1/24 + r/120 + ... in FP32 (|r^4 q4| < 7e-4)
        const float q4 = __fmaf_rn(r.hi, __fmaf_rn(r.hi, __fmaf_rn(r.hi, __fmaf_rn(r.hi, 2.75573192239858907e-06f,
                                                                                   2.48015873015873016e-05f),
                                                               1.98412698412698413e-04f),
                                              1.38888888888888889e-03f),
                                   8.33333333333333333e-03f);
        const float q4b = __fmaf_rn(r.hi, q4, 4.16666666666666667e-02f);
        const df rr2{r2.hi, r2l};
        const df r3 = df_mul(rr2, r);
        const df t3 = df_mul(r3, df{c6_hi, c6_lo});
        const float t4 = __fmul_rn(__fmul_rn(r3.hi, r.hi), q4b);
        em = df_add(df_add(r, df{0.5f * rr2.hi, 0.5f * rr2.lo}), df_add_f(t3, t4));
      }
      // D = 2^n (1 + em) - 1 in double-float
      df D;
      const int ni = (int)n;
      const float pn = ldexpf(1.0f, ni);
      if (ni == 0) {
        D = em;
      } else if (ni <= 24) {
        const df s = two_sum(__fsub_rn(pn, 1.0f), __fmul_rn(pn, em.hi));
        D = fast_two_sum(s.hi, __fmaf_rn(pn, em.lo, s.lo));
      } else {
        const df s = two_sum(pn, __fmul_rn(pn, em.hi));
        D = fast_two_sum(s.hi, __fadd_rn(s.lo, __fmaf_rn(pn, em.lo, -1.0f)));
      }
      // x / D: quotient from an approximate reciprocal, corrected by the fma residual
      // (D.hi > 2^126 only for x > 87, where R < 1e-35 and the reciprocal flushes to 0)
      const float rD = __fdividef(1.0f, D.hi);
      const float q0 = __fmul_rn(xh, rD);
      const float rem = __fadd_rn(__fsub_rn(__fmaf_rn(-q0, D.hi, xh), __fmul_rn(q0, D.lo)), xl);
      return fast_two_sum(q0, __fmul_rn(rem, rD));
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
      df kln;   // scale / ln 2 (log axes): grid cells per unit of ln x
      int n;    // number of grid points
      int log;  // 1: log-spaced
      double scale64, shift64;
    };

    // log2(v) = e + lm for a positive normal v: integer exponent e and |lm| <= 1/2 from log2f of
    // the mantissa scaled into [1/sqrt2, sqrt2).  Absolute error ~3e-8 instead of ~1e-6 for
    // log2f(v) itself when |log2 v| ~ 10 (measured on GB300; __log2f was biased, log2f is not).
    __device__ __forceinline__ void log2_split(float v, float &e, float &lm)
    {
      const int b = __float_as_int(v);
      int ex = ((b >> 23) & 0xff) - 127;
      float m = __int_as_float((b & 0x007fffff) | 0x3f800000);
      if (m > 1.41421356f) {
        m = __fmul_rn(m, 0.5f);
        ex += 1;
      }
      e = (float)ex;
      lm = log2f(m);
    }

    // Cell i in [0, n-2] and fraction in [0, 1] of u = scale * g + shift (u clamped to [0, n-1]),
    // g = log2(v) or v.  u is formed in double-float and its fraction taken before any rounding
    // of u itself: rounding u (up to ~n) to FP32 first costs ~1e-5 of a cell, the largest
    // per-point error of a naive FP32 table lookup.
    // log2(m) for m in [1/sqrt2, sqrt2) as a double-float, absolute error ~5e-10:
    // ln m = 2 atanh(s) = 2 s + 2 s^3 (1/3 + s^2/5 + ... + s^10/13), s = (m-1)/(m+1) in
    // double-float, |s| <= 0.172 (truncation < 1e-11); then times log2(e) in double-float.
    __device__ __forceinline__ df log2_mant_df(float m)
    {
      const float num = __fsub_rn(m, 1.0f);  // exact (Sterbenz)
      const df den = two_sum(m, 1.0f);
      // s = num / den as s0 + s1: s0 from an approximate reciprocal (a few ulp), the residual
      // num - s0 den is exact with an FMA, and s1 = residual / den needs only ~20 bits
      const float r = __fdividef(1.0f, den.hi);
      const float s0 = __fmul_rn(num, r);
      const float rr = __fsub_rn(__fmaf_rn(-s0, den.hi, num), __fmul_rn(s0, den.lo));
      const float s1 = __fmul_rn(rr, r);
      const float t = __fmul_rn(s0, s0);
      float P = __fmaf_rn(t, 7.69230769e-02f, 9.09090909e-02f);  // 1/13, 1/11
      P = __fmaf_rn(t, P, 1.11111111e-01f);                       // 1/9
      P = __fmaf_rn(t, P, 1.42857143e-01f);                       // 1/7
      P = __fmaf_rn(t, P, 2.00000000e-01f);                       // 1/5
      P = __fmaf_rn(t, P, 3.33333343e-01f);                       // 1/3
      const float c3 = __fmul_rn(__fmul_rn(2.0f * s0, t), P);
      const df lnm = fast_two_sum(2.0f * s0, __fmaf_rn(2.0f, s1, c3));
      const df l2e{1.44269502e+00f, 1.92596299e-08f};
      return df_mul(lnm, l2e);
    }

    __device__ __forceinline__ float axis_frac_c(const AxisDev &a, float v, float corr, int &i);
    __device__ __forceinline__ float axis_frac(const AxisDev &a, float v, int &i) { return axis_frac_c(a, v, 0.f, i); }
    __device__ __forceinline__ float frac_from_u(const AxisDev &a, float uh, float ul, int &i);
    // same for a double-float coordinate v = vh + vl, with log2 of the mantissa in double-float
    // (log2_mant_df) and the low part of v entering the index linearly
    __device__ __forceinline__ float axis_frac_df(const AxisDev &a, float vh, float vl, int &i)
    {
      if (!a.log) {
        const df u = df_add(df_mul(a.scale, df_add(df{vh, 0.f}, df{vl, 0.f})), a.shift);
        return frac_from_u(a, u.hi, u.lo, i);
      }
      if (!(vh >= 1e-30f)) {
        vh = 1e-30f;
        vl = 0.f;
      }
      if (!(vh <= 3e38f)) {
        vh = 3e38f;
        vl = 0.f;
      }
      const int b = __float_as_int(vh);
      int ex = ((b >> 23) & 0xff) - 127;
      float m = __int_as_float((b & 0x007fffff) | 0x3f800000);
      if (m > 1.41421356f) {
        m = __fmul_rn(m, 0.5f);
        ex += 1;
      }
      const df lm = log2_mant_df(m);
      // g = ex + lm + vl / (vh ln 2)
      const df g0 = two_sum((float)ex, lm.hi);
      // vl / vh <= 2^-24: an approximate quotient is ample for this first-order term
      const float gl = __fadd_rn(__fadd_rn(g0.lo, lm.lo), __fmul_rn(1.44269504f, __fdividef(vl, vh)));
      const df g = fast_two_sum(g0.hi, gl);
      const df u = df_add(df_mul(a.scale, g), a.shift);
      return frac_from_u(a, u.hi, u.lo, i);
    }
    __device__ __forceinline__ float frac_from_u(const AxisDev &a, float uh, float ul, int &i)
    {
      const float ur = __fadd_rn(uh, ul);
      if (!(ur > 0.f)) {
        i = 0;
        return 0.f;
      }
      if (ur >= (float)(a.n - 1)) {
        i = a.n - 2;
        return 1.f;
      }
      int ii = (int)ur;
      float f = __fadd_rn(__fsub_rn(uh, (float)ii), ul);
      if (f < 0.f) {
        if (ii > 0) {
          ii -= 1;
          f = __fadd_rn(__fsub_rn(uh, (float)ii), ul);
        } else
          f = 0.f;
      }
      if (ii > a.n - 2) {
        ii = a.n - 2;
        f = 1.f;
      }
      i = ii;
      return fminf(f, 1.f);
    }
    // `corr` is added to the low part of u (first-order contribution of a coordinate's low part)
    __device__ __forceinline__ float axis_frac_c(const AxisDev &a, float v, float corr, int &i)
    {
      float uh, ul;
      if (a.log) {
        if (!(v >= 1e-30f)) v = 1e-30f;  // also maps NaN
        if (!(v <= 3e38f)) v = 3e38f;
        float e, lm;
        log2_split(v, e, lm);
        const df p1 = two_prod(a.scale.hi, e);
        const df p2 = two_prod(a.scale.hi, lm);
        const df s1 = two_sum(p1.hi, a.shift.hi);
        const df s2 = two_sum(s1.hi, p2.hi);
        const float lo = __fadd_rn(__fadd_rn(__fadd_rn(p1.lo, p2.lo), __fadd_rn(s1.lo, s2.lo)),
                                   __fadd_rn(__fmaf_rn(a.scale.lo, __fadd_rn(e, lm), 0.f), a.shift.lo));
        uh = s2.hi;
        ul = __fadd_rn(lo, corr);
      } else {
        const df p = two_prod(a.scale.hi, v);
        const df s = two_sum(p.hi, a.shift.hi);
        uh = s.hi;
        ul = __fadd_rn(__fadd_rn(__fadd_rn(p.lo, s.lo), __fmaf_rn(a.scale.lo, v, a.shift.lo)), corr);
      }
      const float ur = __fadd_rn(uh, ul);
      if (!(ur > 0.f)) {
        i = 0;
        return 0.f;
      }
      if (ur >= (float)(a.n - 1)) {
        i = a.n - 2;
        return 1.f;
      }
      int ii = (int)ur;
      float f = __fadd_rn(__fsub_rn(uh, (float)ii), ul);  // uh - ii is exact
      if (f < 0.f) {
        if (ii > 0) {
          ii -= 1;
          f = __fadd_rn(__fsub_rn(uh, (float)ii), ul);
        } else
          f = 0.f;
      }
      if (ii > a.n - 2) {
        ii = a.n - 2;
        f = 1.f;
      }
      i = ii;
      return fminf(f, 1.f);
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
