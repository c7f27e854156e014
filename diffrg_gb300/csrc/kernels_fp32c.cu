// kernels_fp32c.cu -- FP32-compensated persistent kernels for the catalogue workloads.
//
// Structure shared by all kinds (persistent CTAs):
//   * the CTA's dressing tables are staged into shared memory by non-tensor TMA bulk copies
//     (cp.async.bulk + mbarrier complete_tx) and restaged only when an item uses others (S2's
//     accurate form reads its table through mode-interpolated slices formed by k_seg and
//     stages only the cell-centre reciprocals);
//   * work units (item, row range) come from an atomic counter; the node records of the unit's
//     inner axes are TMA-prefetched into a second buffer while the current unit computes;
//   * one thread per row loops over the inner axes on the FP32 pipe with double-float constants,
//     combines with the row's hoisted factor, and the unit is reduced in FP64;
//   * the last unit of an item sums the item's unit partials in a fixed order (deterministic).
// Two arithmetic variants per kind:
//   fast (ACC = false): per-point factors in FP32 and a Kahan sum (~1e-8 of FP64);
//   accurate (ACC = true, GB_PREC_FP32C): coordinate, table fraction and interpolation,
//     regulator, reciprocal, weighted term and row sum in double-float (3e-12 .. 9e-11 of FP64
//     on the benchmark workloads).
// Tensor cores are not used: this is a reduction, not a dense contraction.
#include "device_common.cuh"
#include "integrands.cuh"
#include "kernels.hh"

#include <map>
#include <mutex>
#include <utility>

namespace gbint
{
  using namespace dev;

  namespace
  {
    // A + B*c with A, B, c double-float: one rounding to FP32, or kept as double-float
    __device__ __forceinline__ float lin_df(df A, df B, float c_hi, float c_lo)
    {
      const df p = two_prod(B.hi, c_hi);
      const df s = two_sum(A.hi, p.hi);
      const float corr = __fadd_rn(__fadd_rn(s.lo, A.lo), __fmaf_rn(B.hi, c_lo, __fmaf_rn(B.lo, c_hi, p.lo)));
      return __fadd_rn(s.hi, corr);
    }
    __device__ __forceinline__ df lin_dd(df A, df B, float c_hi, float c_lo)
    {
      const df p = two_prod(B.hi, c_hi);
      const df s = two_sum(A.hi, p.hi);
      const float corr = __fadd_rn(__fadd_rn(s.lo, A.lo), __fmaf_rn(B.hi, c_lo, __fmaf_rn(B.lo, c_hi, p.lo)));
      return fast_two_sum(s.hi, corr);
    }
    // lin_dd without the final renormalisation: the low word stays a few ulp of the high one,
    // which every consumer that takes both words (products, sums, t = x / c - 1) accepts
    __device__ __forceinline__ df lin_du(df A, df B, float c_hi, float c_lo)
    {
      const df p = two_prod(B.hi, c_hi);
      const df s = two_sum(A.hi, p.hi);
      return df{s.hi, __fadd_rn(__fadd_rn(s.lo, A.lo), __fmaf_rn(B.hi, c_lo, __fmaf_rn(B.lo, c_hi, p.lo)))};
    }
    // a + b, the high parts summed exactly and the rest left in the low word (unnormalised)
    __device__ __forceinline__ df df_add_u(df a, df b)
    {
      const df s = two_sum(a.hi, b.hi);
      return df{s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo))};
    }
    __device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }
    __device__ __forceinline__ df df_scale2(df a, float s) { return df{a.hi * s, a.lo * s}; }  // s a power of 2
    __device__ __forceinline__ df dfc(double v) { return df_from(v); }
    __device__ __forceinline__ df df_max(df a, float m) { return a.hi < m ? df{m, 0.f} : a; }

    // fractional index on a linear axis for a double-float coordinate
    __device__ __forceinline__ float axis_frac_lin_df(const AxisDev &a, df v, int &i)
    {
      const df u = df_add(df_mul(a.scale, v), a.shift);
      const float ur = __fadd_rn(u.hi, u.lo);
      if (!(ur > 0.f)) {
        i = 0;
        return 0.f;
      }
      if (ur >= (float)(a.n - 1)) {
        i = a.n - 2;
        return 1.f;
      }
      int ii = (int)floorf(ur);
      float f = __fadd_rn(__fsub_rn(u.hi, (float)ii), u.lo);
      if (f < 0.f) {
        ii -= 1;
        f = __fadd_rn(__fsub_rn(u.hi, (float)ii), u.lo);
      }
      if (ii > a.n - 2) {
        ii = a.n - 2;
        f = 1.f;
      }
      i = ii;
      return fminf(fmaxf(f, 0.f), 1.f);
    }

    __device__ __forceinline__ float rcp32(float x) { return __frcp_rn(x); }

    // Fraction of a double-float coordinate x in cell j of a 1D log table, relative to the cell
    // centre c_j (rc[j] = 1/c_j as hi, lo): f = 1/2 + kln ln(x / c_j) with
    // ln(1+t) = t + t^2 Q(t), t = x/c_j - 1 formed in double-float (p.hi - 1 is exact) and
    // |t| <= sqrt(1.25) - 1 + (one cell when j is off by one near a cell edge); Q is the series
    // through t^9/9, truncation < 3e-10 of a cell.
    // SQ: x is the square of the axis coordinate (1/c_j^2 formed from 1/c_j, half the scale).
    // DEG 6: the series through t^6 (Q through t^4/6), for cells at most 6 % wide (truncation
    // < 1e-10 of a cell within half a cell of the centre)
    template <bool SQ = false, int DEG = 9>
    __device__ __forceinline__ float cell_frac_rr(const AxisDev &a, df rr, df x, df *t_out = nullptr)
    {
      // t = x rr - 1 = th + tl: th = fl(x.hi rr.hi) - 1 is exact (the product lies in [1/2, 2]),
      // tl = the product's rounding error + the cross terms; ln(1 + th + tl) = ln(1 + th) +
      // tl (1 - th) + O(tl^2, th^2 tl)
      const float ph = __fmul_rn(x.hi, rr.hi);
      const float th = __fsub_rn(ph, 1.0f);
      const float tl0 = __fadd_rn(__fmaf_rn(x.hi, rr.hi, -ph), __fmaf_rn(x.hi, rr.lo, __fmul_rn(x.lo, rr.hi)));
      const df t{th, __fmaf_rn(-th, tl0, tl0)};
      if (t_out) *t_out = df{th, tl0};  // x / c_j - 1 itself (the log's correction term aside)
      float Q;
      if constexpr (DEG >= 9) {
        Q = __fmaf_rn(th, 1.11111111e-01f, -1.25e-01f);  // 1/9, -1/8
        Q = __fmaf_rn(th, Q, 1.42857143e-01f);            // 1/7
        Q = __fmaf_rn(th, Q, -1.66666667e-01f);           // -1/6
        Q = __fmaf_rn(th, Q, 2.0e-01f);                   // 1/5
      } else {
        Q = __fmaf_rn(th, -1.66666667e-01f, 2.0e-01f);  // -1/6, 1/5
      }
      Q = __fmaf_rn(th, Q, -2.5e-01f);        // -1/4
      Q = __fmaf_rn(th, Q, 3.33333343e-01f);  // 1/3
      Q = __fmaf_rn(th, Q, -0.5f);
      const float rest = __fmaf_rn(__fmul_rn(th, th), Q, t.lo);  // ln(1+t) = th + rest
      const float kh = SQ ? 0.5f * a.kln.hi : a.kln.hi, kl = SQ ? 0.5f * a.kln.lo : a.kln.lo;
      const float a0 = __fmaf_rn(kh, th, 0.5f);
      return __fadd_rn(a0, __fmaf_rn(kh, rest, __fmul_rn(kl, th)));
    }
    template <bool SQ = false, int DEG = 9>
    __device__ __forceinline__ float cell_frac_at(const AxisDev &a, const float2 *rc, df x, int j, df *t_out = nullptr)
    {
      const float2 r = rc[j];
      df rr{r.x, r.y};
      if constexpr (SQ) rr = df_mul(rr, rr);
      return cell_frac_rr<SQ, DEG>(a, rr, x, t_out);
    }
    // the same fraction as a double-float (its FP32 rounding, ~3e-8 of a cell, is otherwise the
    // largest per-point error of a lookup; used where few points carry an integral)
    __device__ __forceinline__ df cell_frac_at_df(const AxisDev &a, const float2 *rc, df x, int j, df *t_out = nullptr)
    {
      const float2 r = rc[j];
      const df p = df_mul(x, df{r.x, r.y});
      const df t = two_sum(__fsub_rn(p.hi, 1.0f), p.lo);
      if (t_out) *t_out = t;
      const float th = t.hi;
      float Q = __fmaf_rn(th, 1.11111111e-01f, -1.25e-01f);
      Q = __fmaf_rn(th, Q, 1.42857143e-01f);
      Q = __fmaf_rn(th, Q, -1.66666667e-01f);
      Q = __fmaf_rn(th, Q, 2.0e-01f);
      Q = __fmaf_rn(th, Q, -2.5e-01f);
      Q = __fmaf_rn(th, Q, 3.33333343e-01f);
      Q = __fmaf_rn(th, Q, -0.5f);
      const float rest = __fmaf_rn(__fmul_rn(th, th), Q, t.lo);
      const df m = two_prod(a.kln.hi, th);  // kln (th + rest) = m + kln.hi rest + kln.lo th
      const df s0 = two_sum(0.5f, m.hi);
      return fast_two_sum(s0.hi, __fadd_rn(s0.lo, __fadd_rn(m.lo, __fmaf_rn(a.kln.hi, rest, __fmul_rn(a.kln.lo, th)))));
    }
    // cell i and fraction of x on a 1D log table with cell-centre reciprocals (clamped like
    // axis_frac_df): a fast log2 finds the cell to within one, the fraction decides the rest
    // (jt, t): with jt non-null, the cell whose centre t = x / c_jt - 1 refers to (before the
    // off-by-one correction), or -1 where x lies outside the table and was clamped
    template <bool SQ = false, int DEG = 9>
    __device__ __forceinline__ float log_cell_frac(const AxisDev &a, const float2 *rc, df x, int &i, int *jt = nullptr,
                                                   df *t = nullptr)
    {
      const int n = a.n;
      if (jt) *jt = -1;
      if (!(x.hi >= 1e-30f)) x = df{1e-30f, 0.f};  // also maps NaN
      if (!(x.hi <= 3e38f)) x = df{3e38f, 0.f};
      const float ua = __fmaf_rn(SQ ? 0.5f * a.scale.hi : a.scale.hi, __log2f(x.hi), a.shift.hi);
      if (ua < -0.01f) {
        i = 0;
        return 0.f;
      }
      if (ua > (float)(n - 1) + 0.01f) {
        i = n - 2;
        return 1.f;
      }
      int j = min(max((int)floorf(ua), 0), n - 2);
      if (jt) *jt = j;
      float f = cell_frac_at<SQ, DEG>(a, rc, x, j, t);
      if (f < 0.f) {
        if (j > 0) {
          j -= 1;
          f = __fadd_rn(f, 1.f);
        } else
          f = 0.f;
      } else if (f > 1.f) {
        if (j < n - 2) {
          j += 1;
          f = __fsub_rn(f, 1.f);
        } else
          f = 1.f;
      }
      i = j;
      return fminf(fmaxf(f, 0.f), 1.f);
    }
    // cell and double-float fraction on a 1D log table with reciprocals (clamped)
    __device__ __forceinline__ df log_cell_frac_df(const AxisDev &a, const float2 *rc, df x, int &i, int *jt = nullptr,
                                                   df *t = nullptr)
    {
      const int n = a.n;
      if (jt) *jt = -1;
      if (!(x.hi >= 1e-30f)) x = df{1e-30f, 0.f};
      if (!(x.hi <= 3e38f)) x = df{3e38f, 0.f};
      const float ua = __fmaf_rn(a.scale.hi, __log2f(x.hi), a.shift.hi);
      if (ua < -0.01f) {
        i = 0;
        return df{0.f, 0.f};
      }
      if (ua > (float)(n - 1) + 0.01f) {
        i = n - 2;
        return df{1.f, 0.f};
      }
      int j = min(max((int)floorf(ua), 0), n - 2);
      if (jt) *jt = j;
      df f = cell_frac_at_df(a, rc, x, j, t);
      if (f.hi < 0.f) {
        if (j > 0) {
          j -= 1;
          f = df_add_f(f, 1.f);
        } else
          f = df{0.f, 0.f};
      } else if (f.hi > 1.f) {
        if (j < n - 2) {
          j += 1;
          f = df_add_f(f, -1.f);
        } else
          f = df{1.f, 0.f};
      }
      i = j;
      if (f.hi < 0.f) f = df{0.f, 0.f};
      if (f.hi > 1.f) f = df{1.f, 0.f};
      return f;
    }
    // fraction on axis 0 of a table: cell-relative for log axes that carry reciprocals
    __device__ __forceinline__ float frac1_df(const float *T, const TableDev &D, df x, int &i)
    {
      if (D.rc_off && D.rc_axis == 0) return log_cell_frac(D.a0, reinterpret_cast<const float2 *>(T + D.rc_off), x, i);
      return axis_frac_df(D.a0, x.hi, x.lo, i);
    }

    __device__ __forceinline__ float G1_32(const float *T, const AxisDev &a, float x)
    {
      int i;
      const float f = axis_frac(a, x, i);
      return rcp32(__fmaf_rn(lerp32(T[i], T[i + 1], f), x, reg_R(x)));
    }
    // 1 / (z x + R) for double-float z, x, R given as pairs whose low words may exceed half an ulp
    // of the high ones: the product's high part and R's are summed exactly and the rest collects in
    // the low word; the denominator is renormalised once before the reciprocal (one Newton step
    // corrects a low word of a few ulp, not one of 1e-4 of the high word, which an unnormalised
    // regulator can leave after its expansion cancels)
    __device__ __forceinline__ df df_prop(df z, df x, df R)
    {
      const df p = two_prod(z.hi, x.hi);
      const float e = __fadd_rn(p.lo, __fmaf_rn(z.hi, x.lo, __fmul_rn(z.lo, x.hi)));
      const df d0 = two_sum(p.hi, R.hi);
      return df_rcp(fast_two_sum(d0.hi, __fadd_rn(d0.lo, __fadd_rn(e, R.lo))));
    }
    // lerp_df without the final renormalisation (its result feeds df_prop, which takes both words)
    __device__ __forceinline__ df lerp_df_u(float y0, float y1, float f)
    {
      const df d = two_sum(y1, -y0);
      const df p = two_prod(f, d.hi);
      const df s = two_sum(y0, p.hi);
      return df{s.hi, __fadd_rn(s.lo, __fmaf_rn(f, d.lo, p.lo))};
    }
    // R(x) = x / expm1(x) from the Taylor coefficients about the centre of cell j of the table's
    // log axis (3 float4 per cell: a0, a1 as double-float pairs, a2..a7), t = x / c_j - 1:
    // ~30 instructions instead of the exp-based double-float form, no branch on x
    // (SHARED: the coefficients were staged to shared memory)
    template <bool SHARED = false> __device__ __forceinline__ df reg_R_cell(const float4 *rq, int j, df t)
    {
      float4 c0, c1, c2;
      if constexpr (SHARED) {
        c0 = rq[3 * j];
        c1 = rq[3 * j + 1];
        c2 = rq[3 * j + 2];
      } else {
        c0 = __ldg(rq + 3 * j);
        c1 = __ldg(rq + 3 * j + 1);
        c2 = __ldg(rq + 3 * j + 2);
      }
      const float th = t.hi;
      float p = __fmaf_rn(th, c2.y, c2.x);
      p = __fmaf_rn(th, p, c1.w);
      p = __fmaf_rn(th, p, c1.z);
      p = __fmaf_rn(th, p, c1.y);
      p = __fmaf_rn(th, p, c1.x);                                // a2 + a3 t + ... + a7 t^5
      const df q{c0.z, __fmaf_rn(th, p, c0.w)};                  // a1 + t (a2 + ...), unnormalised
      const df tq = two_prod(t.hi, q.hi);                        // a0 + t q, unnormalised
      const df s = two_sum(c0.x, tq.hi);
      return df{s.hi, __fadd_rn(s.lo, __fadd_rn(c0.y, __fadd_rn(tq.lo, __fmaf_rn(t.hi, q.lo, __fmul_rn(t.lo, q.hi)))))};
    }
    // R(x) through the table's cell expansion when x was located by its cell-centre reciprocals
    // and lies inside the table, else the exp-based form
    template <bool EXACT_LOW = false> __device__ __forceinline__ df reg_R_tab(const TableDev &D, int jt, df t, df x)
    {
      if (D.rq_off && jt >= 0) return reg_R_cell(reinterpret_cast<const float4 *>(D.data + D.rq_off), jt, t);
      return reg_R_df<EXACT_LOW>(x);
    }
    __device__ __forceinline__ df G1_df(const float *T, const TableDev &D, df x)
    {
      int i;
      if (D.rc_off && D.rc_axis == 0) {
        int jt;
        df t;
        const float f = log_cell_frac(D.a0, reinterpret_cast<const float2 *>(T + D.rc_off), x, i, &jt, &t);
        return df_prop(lerp_df_u(T[i], T[i + 1], f), x, reg_R_tab(D, jt, t, x));
      }
      const float f = axis_frac_df(D.a0, x.hi, x.lo, i);
      const df z = lerp_df(T[i], T[i + 1], f);
      return df_rcp(df_add(df_mul(z, x), reg_R_df(x)));
    }
    // G(x) with a double-float table fraction (S1: integrals of a few thousand points)
    __device__ __forceinline__ df G1_dff(const float *T, const TableDev &D, df x)
    {
      int i;
      if (D.rc_off && D.rc_axis == 0) {
        int jt;
        df t;
        const df f = log_cell_frac_df(D.a0, reinterpret_cast<const float2 *>(T + D.rc_off), x, i, &jt, &t);
        return df_prop(lerp_dff(T[i], T[i + 1], f), x, reg_R_tab<true>(D, jt, t, x));
      }
      const float f = axis_frac_df(D.a0, x.hi, x.lo, i);
      const df z = lerp_df(T[i], T[i + 1], f);
      return df_rcp(df_add(df_mul(z, x), reg_R_df<true>(x)));
    }
    // a 1D table lookup at a double-float argument, unnormalised (its consumers are products)
    __device__ __forceinline__ df V1_df_u(const float *T, const TableDev &D, df x)
    {
      int i;
      const float f = frac1_df(T, D, x, i);
      return lerp_df_u(T[i], T[i + 1], f);
    }
    // a * b for pairs whose low words may exceed half an ulp, result unnormalised (its consumer
    // takes both words)
    __device__ __forceinline__ df df_mul_u(df a, df b)
    {
      const df p = two_prod(a.hi, b.hi);
      return df{p.hi, __fadd_rn(p.lo, __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi)))};
    }
    __device__ __forceinline__ float V1_32(const float *T, const AxisDev &a, float x)
    {
      int i;
      const float f = axis_frac(a, x, i);
      return lerp32(T[i], T[i + 1], f);
    }
    // z + f dz for a double-float pair (z, dz) packed as {z hi, z lo, dz hi, dz lo}
    __device__ __forceinline__ df lerp_zd(float4 s, float f)
    {
      const df p = two_prod(f, s.z);
      const df t = two_sum(s.x, p.hi);
      return fast_two_sum(t.hi, __fadd_rn(t.lo, __fadd_rn(s.y, __fmaf_rn(f, s.w, p.lo))));
    }
    // bilinear in a row-major [n0][n1] table: lerp along the point-varying axis first and along
    // the fixed one last, so that the rounding of the first lerps is not shared by many points
    // (varying = 0: axis 0 first)
    __device__ __forceinline__ float bil32_v0(const float *d, int n1, int i, float fx, int j, float fy)
    {
      const float *r0 = d + i * n1 + j;
      const float *r1 = r0 + n1;
      return lerp32(lerp32(r0[0], r1[0], fx), lerp32(r0[1], r1[1], fx), fy);
    }
    __device__ __forceinline__ float bil32_v1(const float *d, int n1, int i, float fx, int j, float fy)
    {
      const float *r0 = d + i * n1 + j;
      const float *r1 = r0 + n1;
      return lerp32(lerp32(r0[0], r0[1], fy), lerp32(r1[0], r1[1], fy), fx);
    }
    __device__ __forceinline__ df bil_df_v0(const float *d, int n1, int i, float fx, int j, float fy)
    {
      const float *r0 = d + i * n1 + j;
      const float *r1 = r0 + n1;
      return lerp_dd(lerp_df(r0[0], r1[0], fx), lerp_df(r0[1], r1[1], fx), fy);
    }

    // Double-float running sum of double-float products (accurate form).  A Kahan sum of the high
    // parts loses ~one FP32 rounding of every term (the compensated difference x - c is itself
    // rounded): ~6e-8 per term, ~1e-8 per row and ~3e-10 on a 2048-point integral, measured; the
    // double-float sum keeps ~2^-44 per term.
    // The high parts are summed exactly (two_sum), their rounding errors and the terms' low parts
    // collect in an FP32 low word that is renormalised only when read (it stays ~2^-24 of the
    // sum, so its own rounding is ~2^-48 per term).
    struct AccDF {
      float hi = 0.f, lo = 0.f;
      // add a * b: the product's high part joins the exact sum, its rounding error and cross terms
      // go to the low word (the product is not renormalised first)
      __device__ __forceinline__ void add_prod(df a, df b)
      {
        const df p = two_prod(a.hi, b.hi);
        const float e = __fadd_rn(p.lo, __fmaf_rn(a.hi, b.lo, __fmul_rn(a.lo, b.hi)));
        const df s = two_sum(hi, p.hi);
        hi = s.hi;
        lo = __fadd_rn(lo, __fadd_rn(s.lo, e));
      }
      __device__ __forceinline__ df sum() const { return fast_two_sum(hi, lo); }
      __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
    };

    // bytes of a table's cell-centre reciprocals (staged at the end of its data; 16-byte multiple)
    __device__ __forceinline__ int rc_bytes(const TableDev &T) { return T.rc_off ? T.bytes - 4 * T.rc_off : 0; }
    // S3R staging: a 1D table's propagator records (64 bytes a cell) and its value records
    // (16 bytes a cell, then the difference low words padded to 16 bytes)
    __device__ __forceinline__ int s3r_g_bytes(const TableDev &T) { return 64 * (T.n0 - 1); }
    __device__ __forceinline__ int s3r_rec_bytes(const TableDev &T)
    {
      return 16 * (T.n0 - 1) + (4 * (T.n0 - 1) + 15) / 16 * 16;
    }

    // ---------------------------------------------------------------- per-kind traits
    template <int KIND> struct Traits;
    template <> struct Traits<K_S1> {
      static constexpr int kTables = 1;
    };
    template <> struct Traits<K_S2> {
      static constexpr int kTables = 1;
    };
    template <> struct Traits<K_S3> {
      static constexpr int kTables = 4;
    };
    template <> struct Traits<K_S5> {
      static constexpr int kTables = 2;
    };
    template <> struct Traits<K_S5Z> {
      static constexpr int kTables = 2;
    };
    template <> struct Traits<K_S3R> {
      static constexpr int kTables = 4;
    };

    // node records a unit needs (inner axes), staged back to back
    __device__ __forceinline__ int rec_axes(int kind, const ItemDev &it, int &a0, int &a1)
    {
      switch (kind) {
      case K_S1:
        a0 = 1;
        a1 = -1;
        return it.ax[1].n;
      case K_S2:
      case K_S3:
      case K_S3R:
        a0 = 2;
        a1 = -1;
        return it.ax[2].n;
      case K_S5:
      case K_S5Z:
        a0 = 2;
        a1 = 3;
        return it.ax[2].n + it.ax[3].n;
      }
      a0 = a1 = -1;
      return 0;
    }

    __device__ __forceinline__ void issue_records(int kind, const RunParams &P, int unit, NodeRec *dst,
                                                  uint64_t *bar)
    {
      const UnitDev U = P.units[unit];
      const ItemDev &it = P.items[U.item];
      int a0, a1;
      const int n = rec_axes(kind, it, a0, a1);
      // S5Z: table A's slices at the unit's c1 nodes follow the records (rows ordered (c1, q))
      uint32_t zbytes = 0;
      const float4 *zsrc = nullptr;
      if (kind == K_S5Z) {
        const int nq = it.ax[0].n, ns0 = P.tabs[it.tab[0]].n0 - 1, sl = it.split_log2;
        const int j0 = (U.row_begin >> sl) / nq, j1 = ((U.row_begin + U.row_count - 1) >> sl) / nq;
        zsrc = reinterpret_cast<const float4 *>(P.seg + it.slice_off) + (size_t)j0 * ns0;
        zbytes = (uint32_t)((j1 - j0 + 1) * ns0 * sizeof(float4));
      }
      mbar_expect_tx(bar, (uint32_t)(n * sizeof(NodeRec)) + zbytes);
      tma_bulk_g2s(dst, P.prec + it.ax[a0].off, (uint32_t)(it.ax[a0].n * sizeof(NodeRec)), bar);
      if (a1 >= 0)
        tma_bulk_g2s(dst + it.ax[a0].n, P.prec + it.ax[a1].off, (uint32_t)(it.ax[a1].n * sizeof(NodeRec)), bar);
      if (zbytes) tma_bulk_g2s(dst + n, zsrc, zbytes, bar);
    }

    __device__ __forceinline__ df rec_v(const NodeRec &r) { return df{r.v_hi, r.v_lo}; }
    __device__ __forceinline__ df rec_a(const NodeRec &r) { return df{r.a_hi, r.a_lo}; }
    __device__ __forceinline__ df rec_w(const NodeRec &r) { return df{r.w_hi, r.w_lo}; }
    __device__ __forceinline__ df rec_aw(const NodeRec &r) { return df{r.aw_hi, r.aw_lo}; }

    // ---------------------------------------------------------------- S1: (q, c) x PROP1
    // row = q node i; inner = c nodes; hoisted F_i = w_q kfac G(q^2) Rdot(q^2) (FP64)
    template <bool ACC>
    __device__ __forceinline__ double row_s1(const RunParams &P, const ItemDev &it, int row, const NodeRec *rc,
                                             const float *tab, const TableDev *sT)
    {
      const NodeRec qr = P.prec[it.ax[0].off + row];
      const float4 c = P.aux[it.aux_off];  // p^2, 2p
      const df A = df_add(rec_a(qr), df{c.x, c.y});
      const df B = df_mul(df{c.z, c.w}, rec_v(qr));
      const AxisDev ax = sT[0].a0;
      const int nc = it.ax[1].n;
      if constexpr (!ACC) {
        Kahan k;
#pragma unroll 2
        for (int l = 0; l < nc; ++l) {
          const NodeRec r = rc[l];
          const float x2 = fmaxf(lin_df(A, B, r.v_hi, r.v_lo), 1e-30f);
          const float g = G1_32(tab, ax, x2);
          k.add(__fmaf_rn(r.aw_hi, g, __fmul_rn(r.aw_lo, g)));
        }
        return P.seg[it.seg_off + row] * k.value();
      } else {
        AccDF k;
#pragma unroll 1
        for (int l = 0; l < nc; ++l) {
          const NodeRec r = rc[l];
          const df x2 = df_max(lin_dd(A, B, r.v_hi, r.v_lo), 1e-30f);
          k.add_prod(rec_aw(r), G1_dff(tab, sT[0], x2));
        }
        return P.seg[it.seg_off + row] * k.value();
      }
    }

    // ---------------------------------------------------------------- S2: (mode, q, c) x FTLOOP
    // row = (q node i, c node l); inner = Matsubara modes m, each at +w_m and (m >= pm_from)
    // -w_m.  x2 = |q+p|^2, its |q|-axis table fraction and R(x2) depend on the row only, so they
    // are formed once per row instead of once per mode.  Per point: F_{m,i} G(+-w_m + W, x2)
    // with the hoisted F_{m,i} = w_m w_q Rdot(q^2) G(w_m, q^2) (FP64, kept as a double-float
    // pair) and W the external frequency; the row sum is multiplied by the cos weight.
    template <bool ACC>
    __device__ __forceinline__ double row_s2(const RunParams &P, const ItemDev &it, int row, const NodeRec *rc,
                                             const float *tab, const TableDev *sT)
    {
      const int nc = it.ax[2].n, nq = it.ax[1].n, nm = it.ax[0].n, pmf = it.ax[0].pm_from;
      const int i = row / nc, l = row - i * nc;
      const NodeRec qr = P.prec[it.ax[1].off + i];
      const NodeRec cr = rc[l];
      const float4 *aux = P.aux + it.aux_off;  // p^2, 2p | per (mode, sign): cell, fraction, w^2
      const float4 c = aux[0];
      const df A = df_add(rec_a(qr), df{c.x, c.y});
      const df B = df_mul(df{c.z, c.w}, rec_v(qr));
      const TableDev &Z = sT[0];
      const int n1 = Z.n1;
      // With W = 0 the +-w_m evaluations read |w| and w^2 only: they are bitwise equal, so one
      // evaluation is doubled (exact) instead of computing the second.
      const bool twin = it.args[3] == 0.0;
      const float2 *F = reinterpret_cast<const float2 *>(P.seg + it.seg_off) + i;  // F_{m,i} at [m * nq]
      if constexpr (!ACC) {
        const float x2 = fmaxf(lin_df(A, B, cr.v_hi, cr.v_lo), 1e-30f);
        int jq;
        float fq;
        if (Z.a1.log) {
          AxisDev axq = Z.a1;  // log |q| axis fed with x2 = |q+p|^2: half the log2 scale
          axq.scale.hi *= 0.5f;
          axq.scale.lo *= 0.5f;
          fq = axis_frac(axq, x2, jq);
        } else {
          fq = axis_frac(Z.a1, __fsqrt_rn(x2), jq);  // linear |q| axis: the root itself
        }
        const float R = reg_R(x2);
        Kahan k;
#pragma unroll 1
        for (int m = 0; m < nm; ++m) {
          const float4 r0 = aux[1 + 2 * m];
          float g = rcp32(__fmaf_rn(bil32_v1(tab, n1, __float_as_int(r0.x), r0.y, jq, fq),
                                    __fadd_rn(__fadd_rn(r0.z, x2), r0.w), R));
          if (m >= pmf) {
            if (twin) {
              g = __fadd_rn(g, g);
            } else {
              const float4 r1 = aux[2 + 2 * m];
              g = __fadd_rn(g, rcp32(__fmaf_rn(bil32_v1(tab, n1, __float_as_int(r1.x), r1.y, jq, fq),
                                               __fadd_rn(__fadd_rn(r1.z, x2), r1.w), R)));
            }
          }
          const float2 f = F[(size_t)m * nq];
          k.add(__fmaf_rn(f.x, g, __fmul_rn(f.y, g)));
        }
        return (double)df_round(rec_w(cr)) * k.value();
      } else {
        // cell-centre reciprocals of the |q| axis (fed with |q+p|^2), when the table has them
        // (staged alone, at the start of this table's shared-memory block)
        const float2 *rcq = (Z.rc_off && Z.rc_axis == 1 && Z.rc_sq) ? reinterpret_cast<const float2 *>(tab) : nullptr;
        const df x2 = df_max(lin_dd(A, B, cr.v_hi, cr.v_lo), 1e-30f);
        int jq;
        float fq;
        if (rcq) {
          fq = log_cell_frac<true>(Z.a1, rcq, x2, jq);
        } else if (Z.a1.log) {
          AxisDev axq = Z.a1;  // log |q| axis fed with x2 = |q+p|^2: half the log2 scale
          axq.scale.hi *= 0.5f;
          axq.scale.lo *= 0.5f;
          fq = axis_frac_df(axq, x2.hi, x2.lo, jq);
        } else {
          const df qa = df_sqrt(x2);  // linear |q| axis: the root itself
          fq = axis_frac_df(Z.a1, qa.hi, qa.lo, jq);
        }
        const df R = reg_R_df(x2);
        // The table interpolated along its mode axis at every (mode, sign) frequency of this
        // item was formed per |q| cell in FP64 (segment SEG_S2Z): {z, dz} at [record * (n1 - 1)
        // + cell], so a point lerps along |q| only.  Records are (mode m, sign) = 2 m, 2 m + 1.
        const int ns = n1 - 1, zstep = 2 * ns;
        const float4 *zp = reinterpret_cast<const float4 *>(P.seg + it.slice_off) + jq;  // record 2 m
        const float2 *wp = reinterpret_cast<const float2 *>(aux + 1) + 1;  // its w^2 (record r at [2 r])
        const float2 *fp = F;                                              // F_{m,i}, stride nq
        // G = 1 / (z (w^2 + x2) + R) with the intermediate pairs left unnormalised (their low words
        // stay a few ulp of the high ones; the products and the reciprocal's residual take both
        // words, so only the renormalising additions are saved)
        const auto G = [&](const float4 &zs, const float2 &w2) {
          const df zp = two_prod(fq, zs.z);  // z = zs.x + fq dz: exact high sum, low word collected
          const df zt = two_sum(zs.x, zp.hi);
          const df z{zt.hi, __fadd_rn(zt.lo, __fadd_rn(zs.y, __fmaf_rn(fq, zs.w, zp.lo)))};
          const df s0 = two_sum(w2.x, x2.hi);  // s = w^2 + x2
          const float sl = __fadd_rn(s0.lo, __fadd_rn(w2.y, x2.lo));
          const df p = two_prod(z.hi, s0.hi);  // D = z s + R
          const float e = __fadd_rn(p.lo, __fmaf_rn(z.hi, sl, __fmul_rn(z.lo, s0.hi)));
          const df d0 = two_sum(p.hi, R.hi);
          return df_rcp(df{d0.hi, __fadd_rn(d0.lo, __fadd_rn(e, R.lo))});
        };
        AccDF k1, k2;  // modes with one sign (below pm_from); modes with both signs
        const int m1 = min(pmf, nm);
#pragma unroll 1
        for (int m = 0; m < m1; ++m) {
          const float2 f = __ldg(fp);
          k1.add_prod(df{f.x, f.y}, G(__ldg(zp), __ldg(wp)));
          zp += zstep;
          wp += 4;
          fp += nq;
        }
        if (m1 < nm) {
          // the slice, w^2 and hoisted factor of the next mode are loaded one iteration ahead
          // (L1/L2 latency would otherwise stall every mode); two modes per loop body interleave
          // their independent double-float chains
          float4 zn = __ldg(zp);
          float2 wn = __ldg(wp), fn = __ldg(fp);
          if (twin) {
            // W = 0: the two signs read |w| and w^2 only and are bitwise equal, so each mode is
            // evaluated once and the sum doubled (exact) at the end
#pragma unroll 2
            for (int m = m1; m < nm; ++m) {
              const float4 z = zn;
              const float2 w2 = wn, f = fn;
              if (m + 1 < nm) {
                zp += zstep;
                wp += 4;
                fp += nq;
                zn = __ldg(zp);
                wn = __ldg(wp);
                fn = __ldg(fp);
              }
              k2.add_prod(df{f.x, f.y}, G(z, w2));
            }
            k2.hi *= 2.f;
            k2.lo *= 2.f;
          } else {
            float4 zn1 = __ldg(zp + ns);
            float2 wn1 = __ldg(wp + 2);
#pragma unroll 1
            for (int m = m1; m < nm; ++m) {
              const float4 z = zn, z1 = zn1;
              const float2 w2 = wn, w21 = wn1, f = fn;
              if (m + 1 < nm) {
                zp += zstep;
                wp += 4;
                fp += nq;
                zn = __ldg(zp);
                zn1 = __ldg(zp + ns);
                wn = __ldg(wp);
                wn1 = __ldg(wp + 2);
                fn = __ldg(fp);
              }
              k2.add_prod(df{f.x, f.y}, df_add(G(z, w2), G(z1, w21)));
            }
          }
        }
        const df ksum = df_add(k1.sum(), k2.sum());
        const df row_sum = df_mul(rec_w(cr), ksum);
        return (double)row_sum.hi + (double)row_sum.lo;
      }
    }

    // ---------------------------------------------------------------- S3: (q, c, phi) x PROP3
    // row = (q node i, c node j); inner = phi nodes; hoisted F_i = w_q Rdot(q^2) G_A(q^2) (FP64)
    template <bool ACC>
    // part / nsplit: this call sums the phi nodes l = part, part + nsplit, ... of the row
    __device__ __forceinline__ double row_s3(const RunParams &P, const ItemDev &it, int row, int part, int nsplit,
                                             const NodeRec *rc, const float *tab, const TableDev *sT,
                                             const int *toff)
    {
      const int nc = it.ax[1].n;
      const int i = row / nc, j = row - i * nc;
      const NodeRec qr = P.prec[it.ax[0].off + i];
      const NodeRec cr = P.prec[it.ax[1].off + j];
      const float4 *aux = P.aux + it.aux_off;  // (P, cos th), (P^2, P^2/4), (sin th, -)
      const float4 c0 = aux[0], c1 = aux[1], c2 = aux[2];
      const df q2 = rec_a(qr);
      const df qP = df_mul(rec_v(qr), df{c0.x, c0.y});
      const df X = df_mul(qP, df_mul(rec_v(cr), df{c0.z, c0.w}));  // q P c cos(th)
      const df q2pp = df_add(q2, df{c1.x, c1.y});
      const df A = df_add(q2pp, df_scale2(df_neg(X), 2.f));  // |q-p|^2 at cos(phi) = 0
      const df Ap = df_add(df_add(q2, df{c1.z, c1.w}), df_neg(X));
      const df B = df_scale2(df_neg(df_mul(qP, df_mul(rec_a(cr), df{c2.x, c2.y}))), 2.f);  // -2 q P s sin(th)
      const df Bh = df_scale2(B, 0.5f);
      const df third = dfc(1.0 / 3.0);
      const df sbd = df_mul(q2pp, third);
      const float *TB = tab + toff[1], *TC = tab + toff[2], *TD = tab + toff[3];
      const AxisDev aB = sT[1].a0, aC = sT[2].a0, aD = sT[3].a0;
      const int nf = it.ax[2].n;
      // The integrand reads phi only through cos(phi), and the phi rule is symmetric
      // (phi_l + phi_{n-1-l} = 2 pi, equal weights): the first half of the nodes is summed with
      // doubled weights (the middle node of an odd rule once).
      const int nh = (nf + 1) >> 1;
      double inner;
      if constexpr (!ACC) {
        const float sb = df_round(sbd);
        Kahan k;
#pragma unroll 1
        for (int l = part; l < nh; l += nsplit) {
          const NodeRec r = rc[l];  // a = cos(phi), w = 2 pi w_phi
          const float r2 = fmaxf(lin_df(A, B, r.a_hi, r.a_lo), 1e-30f);
          const float t2 = fmaxf(lin_df(Ap, Bh, r.a_hi, r.a_lo), 1e-30f);
          const float sv = __fmaf_rn(r2, third.hi, __fmaf_rn(r2, third.lo, sb));
          const float g = G1_32(TB, aB, r2) * V1_32(TC, aC, sv) * V1_32(TD, aD, t2);
          const float ws = 2 * l + 1 == nf ? 1.f : 2.f;
          k.add(__fmaf_rn(ws * r.w_hi, g, __fmul_rn(ws * r.w_lo, g)));
        }
        inner = k.value();
      } else {
        AccDF k;
#pragma unroll 1
        for (int l = part; l < nh; l += nsplit) {
          const NodeRec r = rc[l];
          const df r2 = df_max(lin_dd(A, B, r.a_hi, r.a_lo), 1e-30f);
          const df t2 = df_max(lin_dd(Ap, Bh, r.a_hi, r.a_lo), 1e-30f);
          const df sv = df_add(sbd, df_mul(r2, third));
          const df g = df_mul_u(df_mul_u(G1_df(TB, sT[1], r2), V1_df_u(TC, sT[2], sv)), V1_df_u(TD, sT[3], t2));
          k.add_prod(df_scale2(rec_w(r), 2 * l + 1 == nf ? 1.f : 2.f), g);
        }
        inner = k.value();
      }
      return P.seg[it.seg_off + i] * P.pw[it.ax[1].off + j] * inner;
    }

    // ---------------------------------------------------------------- S3R: S3 through cell records
    // The accurate S3 with its three point-dependent tables (B at r2 = |q-p|^2, C at
    // s = (q^2 + p^2 + r2)/3, D at t2 = |q-p/2|^2) read through per-cell records staged in shared
    // memory.  C's and D's value records: one 16-byte load gives a cell's reciprocal, value and
    // difference (split exactly into two floats, so the lerp needs no two_sum of the endpoints).
    // B's propagator records: 1 / (Z(x) x + R(x)) as the cell's series sum g_k t^k, t = x / c_j - 1,
    // through t^8 (k_cell_records) -- no fraction, lerp, regulator or reciprocal for B per point.
    // t2 follows from r2 (t2 = r2/2 + q^2/2 - P^2/4).  Staged layout (floats): toff[1] B's
    // propagator records (16 a cell), toff[2], toff[3] the value records of C and D, then their
    // difference low words.
    struct RecTab {
      const float4 *rec;
      const float *dlo;
    };
    __device__ __forceinline__ RecTab rec_tab(const float *tab, int off, int cells)
    {
      return RecTab{reinterpret_cast<const float4 *>(tab + off), tab + off + 4 * cells};
    }
    // cells at most 6 % wide: the short series of cell_frac_rr applies
    __device__ __forceinline__ bool narrow_cells(const AxisDev &a) { return a.scale.hi >= 11.9f; }
    // cell j and fraction of x (x.hi > 0 or NaN; NaN lands in a clamped cell) on a record table,
    // clamped like log_cell_frac; r = the record of cell j; (jt, t): the cell whose centre t =
    // x / c_jt - 1 refers to, or jt = -1 where x lies outside the table.  DEG 6 (cells at most
    // 6 % wide): the short series is exact to ~1e-11 of a cell for x inside cell jt; the few
    // points the fast log2 puts one cell off (within ~2e-6 of a cell edge, so |t| up to 1.5
    // cells) get a fraction good to ~1e-7 of a cell before the shift by one, which moves their
    // value by < 1e-8 relative -- a few in a million points, below 1e-13 of an integral.
    template <int DEG>
    __device__ __forceinline__ float rec_cell_frac(const AxisDev &a, const RecTab &T, df x, int &j, float4 &r, int &jt,
                                                   df &t)
    {
      const int n = a.n;
      jt = -1;
      const float ua = __fmaf_rn(a.scale.hi, __log2f(x.hi), a.shift.hi);
      if (ua < -0.01f) {
        j = 0;
        r = T.rec[0];
        return 0.f;
      }
      if (ua > (float)(n - 1) + 0.01f) {
        j = n - 2;
        r = T.rec[n - 2];
        return 1.f;
      }
      j = min((int)ua, n - 2);  // ua >= -0.01 here: truncation gives the cell (NaN converts to 0)
      jt = j;
      r = T.rec[j];
      float f = cell_frac_rr<false, DEG>(a, df{r.x, r.y}, x, &t);
      if (f < 0.f) {
        if (j > 0) {
          j -= 1;
          f = __fadd_rn(f, 1.f);
          r = T.rec[j];
        } else
          f = 0.f;
      } else if (f > 1.f) {
        if (j < n - 2) {
          j += 1;
          f = __fsub_rn(f, 1.f);
          r = T.rec[j];
        } else
          f = 1.f;
      }
      return fminf(fmaxf(f, 0.f), 1.f);
    }
    // y_j + f (y_{j+1} - y_j) from a record, unnormalised (the same operations as lerp_df_u)
    __device__ __forceinline__ df rec_lerp_u(const float4 &r, float dlo, float f)
    {
      const df p = two_prod(f, r.w);
      const df s = two_sum(r.z, p.hi);
      return df{s.hi, __fadd_rn(s.lo, __fmaf_rn(f, dlo, p.lo))};
    }
    template <int DEG> __device__ __forceinline__ df V1_rec(const RecTab &T, const AxisDev &a, df x)
    {
      int j, jt;
      float4 r;
      df t;
      const float f = rec_cell_frac<DEG>(a, T, x, j, r, jt, t);
      return rec_lerp_u(r, T.dlo[j], f);
    }
    // t = x rr - 1 as a normalised double-float: fl(x.hi rr.hi) - 1 is exact (see cell_frac_rr),
    // the product's rounding error and cross terms (~1e-7) join it by fast_two_sum, so that the
    // low word left for the series' first-order terms is ~1e-9
    __device__ __forceinline__ df rec_t(df x, float rh, float rl)
    {
      const float ph = __fmul_rn(x.hi, rh);
      const float th = __fsub_rn(ph, 1.0f);
      return fast_two_sum(th, __fadd_rn(__fmaf_rn(x.hi, rh, -ph), __fmaf_rn(x.hi, rl, __fmul_rn(x.lo, rh))));
    }
    // 1 / (Z(x) x + R(x)) on B from its propagator records G (four float4 arrays of n - 1 cells:
    // {1/c_j hi, lo, g0 hi, lo}, {g1 hi, lo, g2 hi, lo}, {g3, g4, g5, g6}, {g7, g8, el, +-eh}).  The fast log2
    // that picks cell j is off by up to ~3e-5 of a cell, so a t beyond the cell's edges moved in
    // by 4e-7 (el, eh) is placed exactly (FP64 against the table's edges e_lo, e_hi).  Outside
    // the table, or in a cell whose series is not trusted (eh < 0), the value records, the
    // regulator expansion and a reciprocal from global memory (TBg, rqg) give the propagator.
    template <int DEG>
    __device__ __forceinline__ df G1_grec(const float4 *G, const TableDev &T, const RecTab &TBg, const float4 *rqg,
                                          df x)
    {
      const AxisDev &a = T.a0;
      const int n = a.n;
      const float ua = __fmaf_rn(a.scale.hi, __log2f(x.hi), a.shift.hi);
      if (ua >= 0.f && ua <= (float)(n - 1)) {
        const int nc = n - 1;
        int j = min((int)ua, n - 2);
        float4 c0 = G[j], c3 = G[3 * nc + j];
        df t = rec_t(x, c0.x, c0.y);
        bool in = true;
        if (t.hi <= c3.z || t.hi >= fabsf(c3.w)) {
          const double td = (double)t.hi + (double)t.lo;
          const int jn = td > T.e_hi ? j + 1 : (td < T.e_lo ? j - 1 : j);
          if (jn != j) {
            in = jn >= 0 && jn <= n - 2;
            if (in) {
              j = jn;
              c0 = G[j];
              c3 = G[3 * nc + j];
              t = rec_t(x, c0.x, c0.y);
            }
          }
        }
        if (in && c3.w > 0.f) {
          const float4 c1 = G[nc + j], c2 = G[2 * nc + j];
          const float th = t.hi;
          float S = __fmaf_rn(th, c3.y, c3.x);  // g7 + t g8
          S = __fmaf_rn(th, S, c2.w);
          S = __fmaf_rn(th, S, c2.z);
          S = __fmaf_rn(th, S, c2.y);
          S = __fmaf_rn(th, S, c2.x);  // g3 + t (g4 + ...)
          // P = g2 + t S, normalised (so are Q and the result: the unnormalised products
          // downstream drop lo x lo)
          const df P = fast_two_sum(c1.z, __fmaf_rn(th, S, c1.w));
          const df tp = two_prod(th, P.hi);  // Q = g1 + t P
          const df q = two_sum(c1.x, tp.hi);
          const float ql =
              __fadd_rn(q.lo, __fadd_rn(c1.y, __fadd_rn(tp.lo, __fmaf_rn(th, P.lo, __fmul_rn(t.lo, P.hi)))));
          const df tq = two_prod(th, q.hi);  // g0 + t Q
          const df s = two_sum(c0.z, tq.hi);
          return df{s.hi, __fadd_rn(s.lo, __fadd_rn(c0.w, __fadd_rn(tq.lo, __fmaf_rn(th, ql, __fmul_rn(t.lo, q.hi)))))};
        }
      }
      int j, jt;
      float4 r;
      df t;
      const float f = rec_cell_frac<DEG>(a, TBg, x, j, r, jt, t);
      const df R = jt >= 0 ? reg_R_cell<false>(rqg, jt, t) : reg_R_df(x);
      return df_prop(rec_lerp_u(r, TBg.dlo[j], f), x, R);
    }
    // part / nsplit: this call sums the phi nodes l = part, part + nsplit, ... of the row
    __device__ __forceinline__ double row_s3r(const RunParams &P, const ItemDev &it, int row, int part, int nsplit,
                                              const NodeRec *rc, const float *tab, const TableDev *sT,
                                              const int *toff)
    {
      const int nc = it.ax[1].n;
      const int i = row / nc, j = row - i * nc;
      const NodeRec qr = P.prec[it.ax[0].off + i];
      const NodeRec cr = P.prec[it.ax[1].off + j];
      const float4 *aux = P.aux + it.aux_off;  // (P, cos th), (P^2, P^2/4), (sin th, -)
      const float4 c0 = aux[0], c1 = aux[1], c2 = aux[2];
      const df q2 = rec_a(qr);
      const df qP = df_mul(rec_v(qr), df{c0.x, c0.y});
      const df X = df_mul(qP, df_mul(rec_v(cr), df{c0.z, c0.w}));  // q P c cos(th)
      const df q2pp = df_add(q2, df{c1.x, c1.y});
      const df A = df_add(q2pp, df_scale2(df_neg(X), 2.f));  // |q-p|^2 at cos(phi) = 0
      const df B = df_scale2(df_neg(df_mul(qP, df_mul(rec_a(cr), df{c2.x, c2.y}))), 2.f);  // -2 q P s sin(th)
      const df Ct = df_add(df_scale2(q2, 0.5f), df_neg(df{c1.z, c1.w}));  // t2 - r2 / 2
      const df third = dfc(1.0 / 3.0);
      const df sbd = df_mul(q2pp, third);
      const AxisDev aB = sT[1].a0, aC = sT[2].a0, aD = sT[3].a0;
      const float4 *GB = reinterpret_cast<const float4 *>(tab + toff[1]);
      const RecTab TC = rec_tab(tab, toff[2], sT[2].n0 - 1), TD = rec_tab(tab, toff[3], sT[3].n0 - 1);
      const RecTab TBg = rec_tab(sT[1].data, sT[1].cr_off, sT[1].n0 - 1);
      const float4 *rqB = reinterpret_cast<const float4 *>(sT[1].data + sT[1].rq_off);
      const int nf = it.ax[2].n;
      // the phi rule is symmetric and the integrand reads phi through cos(phi) only (see row_s3)
      const int nh = (nf + 1) >> 1;
      auto phi_loop = [&](auto deg) {
        constexpr int DEG = decltype(deg)::value;
        AccDF k;
#pragma unroll 1
        for (int l = part; l < nh; l += nsplit) {
          const NodeRec r = rc[l];  // a = cos(phi), w = 2 pi w_phi
          // r2, t2 and s unnormalised (their lookups take both words)
          const df r2 = df_max(lin_du(A, B, r.a_hi, r.a_lo), 1e-30f);
          const df t2 = df_max(df_add_u(df_scale2(r2, 0.5f), Ct), 1e-30f);
          const df sv = df_add_u(sbd, df_mul_u(r2, third));
          const df g =
              df_mul_u(df_mul_u(G1_grec<DEG>(GB, sT[1], TBg, rqB, r2), V1_rec<DEG>(TC, aC, sv)), V1_rec<DEG>(TD, aD, t2));
          k.add_prod(df_scale2(rec_w(r), 2 * l + 1 == nf ? 1.f : 2.f), g);
        }
        return k.value();
      };
      // the short series when all three tables have cells at most 6 % wide (one branch per row,
      // the same for every thread of a unit)
      const double inner = (narrow_cells(aB) && narrow_cells(aC) && narrow_cells(aD))
                               ? phi_loop(std::integral_constant<int, 6>{})
                               : phi_loop(std::integral_constant<int, 9>{});
      return P.seg[it.seg_off + i] * P.pw[it.ax[1].off + j] * inner;
    }

    // ---------------------------------------------------------------- S5: (q, c1, c2, phi) x VERT4
    // row = (q node i, c1 node j); mid = c2 nodes; inner = phi nodes;
    // hoisted F_ij = w_q w_c1 Rdot(q^2) G(q^2, c1) (FP64)
    template <bool ACC>
    __device__ __forceinline__ double row_s5(const RunParams &P, const ItemDev &it, int row, const NodeRec *rc,
                                             const float *tab, const TableDev *sT, const int *toff)
    {
      const int n1 = it.ax[1].n;
      const int i = row / n1, j = row - i * n1;
      const NodeRec qr = P.prec[it.ax[0].off + i];
      const NodeRec cr = P.prec[it.ax[1].off + j];
      const float4 *aux = P.aux + it.aux_off;  // (P, P^2), (cos a, sin a)
      const float4 k0 = aux[0], k1 = aux[1];
      const df qP = df_mul(rec_v(qr), df{k0.x, k0.y});
      const df q2pp = df_add(rec_a(qr), df{k0.z, k0.w});
      const df c1 = rec_v(cr);
      const df qPc1 = df_mul(qP, c1);
      const df r1d = df_max(df_add(q2pp, df_scale2(df_neg(qPc1), 2.f)), 1e-30f);  // |q-p1|^2
      const df A2 = df_add(q2pp, df_scale2(df_mul(qPc1, df{k1.x, k1.y}), 2.f));
      const df B2 = df_scale2(df_mul(qP, df_mul(rec_a(cr), df{k1.z, k1.w})), 2.f);
      const TableDev &TA = sT[0];
      const float *DA = tab + toff[0], *DB = tab + toff[1];
      const int tn1 = TA.n1;
      int jc1;
      const float fc1 = axis_frac_lin_df(TA.a1, c1, jc1);
      const int n2 = it.ax[2].n, n3 = it.ax[3].n;
      // the inner integrand reads phi only through cos(phi) and the phi rule is symmetric: the
      // first half of the nodes with doubled weights (the middle node of an odd rule once)
      const int nh3 = (n3 + 1) >> 1;
      const NodeRec *rphi = rc + n2;
      if constexpr (!ACC) {
        const float r1 = df_round(r1d);
        int ir1;
        const float fr1 = axis_frac(TA.a0, r1, ir1);
        const float Rr1 = reg_R(r1);
        Kahan kmid;
#pragma unroll 1
        for (int l = 0; l < n2; ++l) {
          const NodeRec r2r = rc[l];  // c2: v = c2, a = s2, w = 2 w_c2
          int jc2;
          const float fc2 = axis_frac_lin_df(TA.a1, rec_v(r2r), jc2);
          const float gr1 = rcp32(__fmaf_rn(bil32_v0(DA, tn1, ir1, fr1, jc2, fc2), r1, Rr1));
          const df Bs = df_mul(B2, rec_a(r2r));
          Kahan kin;
#pragma unroll 2
          for (int m = 0; m < nh3; ++m) {
            const NodeRec rp = rphi[m];  // a = cos(phi), w = 2 pi w_phi
            const float x = fmaxf(lin_df(A2, Bs, rp.a_hi, rp.a_lo), 1e-30f);
            int ix;
            const float fx = axis_frac(TA.a0, x, ix);
            const float gv = rcp32(__fmaf_rn(bil32_v0(DA, tn1, ix, fx, jc1, fc1), x, reg_R(x)));
            const float g = gv * bil32_v0(DB, tn1, ix, fx, jc2, fc2);
            const float ws = 2 * m + 1 == n3 ? 1.f : 2.f;
            kin.add(__fmaf_rn(ws * rp.w_hi, g, __fmul_rn(ws * rp.w_lo, g)));
          }
          const float mt = __fmul_rn((float)kin.value(), gr1);
          kmid.add(__fmaf_rn(r2r.w_hi, mt, __fmul_rn(r2r.w_lo, mt)));
        }
        return P.seg[it.seg_off + row] * kmid.value();
      } else {
        int ir1;
        const float fr1 = frac1_df(DA, TA, r1d, ir1);
        const df Rr1 = reg_R_df(r1d);
        AccDF kmid;
#pragma unroll 1
        for (int l = 0; l < n2; ++l) {
          const NodeRec r2r = rc[l];
          int jc2;
          const float fc2 = axis_frac_lin_df(TA.a1, rec_v(r2r), jc2);
          const df gr1 = df_rcp(df_add(df_mul(bil_df_v0(DA, tn1, ir1, fr1, jc2, fc2), r1d), Rr1));
          const df Bs = df_mul(B2, rec_a(r2r));
          AccDF kin;
#pragma unroll 1
          for (int m = 0; m < nh3; ++m) {
            const NodeRec rp = rphi[m];
            const df x = df_max(lin_dd(A2, Bs, rp.a_hi, rp.a_lo), 1e-30f);
            int ix;
            const float fx = frac1_df(DA, TA, x, ix);
            const df gv = df_rcp(df_add(df_mul(bil_df_v0(DA, tn1, ix, fx, jc1, fc1), x), reg_R_df(x)));
            const df g = df_mul(gv, bil_df_v0(DB, tn1, ix, fx, jc2, fc2));
            kin.add_prod(df_scale2(rec_w(rp), 2 * m + 1 == n3 ? 1.f : 2.f), g);
          }
          const df si = kin.sum();
          kmid.add_prod(rec_w(r2r), df_mul(si, gr1));
        }
        return P.seg[it.seg_off + row] * kmid.value();
      }
    }

    // ---------------------------------------------------------------- S5Z: S5 through table slices
    // The accurate S5 with tables A and B interpolated along their cos axis once per step (k_seg,
    // SEG_AX1, FP64, {z, dz} double-float pairs per |q-p|^2 cell): A at the c1 nodes (this unit's
    // rows, staged after the node records), B at the c2 nodes (read through L1: staging them
    // too would hold a CTA's shared memory at ~180 KB and halve the resident warps, measured 13 %
    // slower), A at the c2 nodes (through L1, once per (row, c2)).  A point then lerps along the
    // |q-p|^2 axis only, twice, instead of two double-float bilinears.
    // row = (c1 node j, q node i), q fastest, so a unit spans few c1 nodes.
    // part / nsplit: this call sums the c2 nodes l = part, part + nsplit, ... of the row.
    // DEG: terms of the cell fraction's ln series (6 when table A's cells are at most 6 % wide,
    // see rec_cell_frac for the points one cell off)
    template <int DEG>
    __device__ __forceinline__ double row_s5z(const RunParams &P, const ItemDev &it, int row, int row0, int part,
                                              int nsplit, const NodeRec *rc, const float *tab, const TableDev *sT)
    {
      const int nq = it.ax[0].n, n1 = it.ax[1].n;
      const int j = row / nq, i = row - j * nq;
      const NodeRec qr = P.prec[it.ax[0].off + i];
      const NodeRec cr = P.prec[it.ax[1].off + j];
      const float4 *aux = P.aux + it.aux_off;  // (P, P^2), (cos a, sin a)
      const float4 k0 = aux[0], k1 = aux[1];
      const df qP = df_mul(rec_v(qr), df{k0.x, k0.y});
      const df q2pp = df_add(rec_a(qr), df{k0.z, k0.w});
      const df c1 = rec_v(cr);
      const df qPc1 = df_mul(qP, c1);
      const df r1d = df_max(df_add(q2pp, df_scale2(df_neg(qPc1), 2.f)), 1e-30f);  // |q-p1|^2
      const df A2 = df_add(q2pp, df_scale2(df_mul(qPc1, df{k1.x, k1.y}), 2.f));
      const df B2 = df_scale2(df_mul(qP, df_mul(rec_a(cr), df{k1.z, k1.w})), 2.f);
      const TableDev &TA = sT[0];
      const int ns0 = TA.n0 - 1;
      // table A's cell-centre reciprocals (staged first) give the |q-p|^2 cell and fraction
      const float2 *rca = (TA.rc_off && TA.rc_axis == 0) ? reinterpret_cast<const float2 *>(tab) : nullptr;
      // the |q-p|^2 fraction, and with it the cell and t = x / c - 1 the regulator expansion uses
      auto frac0 = [&](df x, int &ix, int &jt, df &t) -> float {
        jt = -1;
        return rca ? log_cell_frac<false, DEG>(TA.a0, rca, x, ix, &jt, &t) : axis_frac_df(TA.a0, x.hi, x.lo, ix);
      };
      const float4 *zb = reinterpret_cast<const float4 *>(P.seg + it.slice_off2);  // B at c2 node l: [l * ns0]
      const int n2 = it.ax[2].n, n3 = it.ax[3].n;
      const float4 *za = reinterpret_cast<const float4 *>(rc + n2 + n3) + (j - row0 / nq) * ns0;  // A at c1 node j
      const float4 *za2 = reinterpret_cast<const float4 *>(P.seg + it.slice_off3);  // A at c2 node l: [l * ns0]
      const int nh3 = (n3 + 1) >> 1;
      const NodeRec *rphi = rc + n2;
      int ir1, jr1;
      df tr1;
      const float fr1 = frac0(r1d, ir1, jr1, tr1);
      const df Rr1 = reg_R_tab(TA, jr1, tr1, r1d);
      AccDF kmid;
#pragma unroll 1
      for (int l = part; l < n2; l += nsplit) {
        const NodeRec r2r = rc[l];  // c2: v = c2, a = s2, w = 2 w_c2
        const df gr1 = df_rcp(df_add(df_mul(lerp_zd(__ldg(za2 + (size_t)l * ns0 + ir1), fr1), r1d), Rr1));
        const df Bs = df_mul(B2, rec_a(r2r));
        const float4 *zbl = zb + l * ns0;
        AccDF kin;
#pragma unroll 1
        for (int m = 0; m < nh3; ++m) {
          const NodeRec rp = rphi[m];
          const df x = df_max(lin_du(A2, Bs, rp.a_hi, rp.a_lo), 1e-30f);  // unnormalised: see lin_du
          int ix, jx;
          df tx;
          const float fx = frac0(x, ix, jx, tx);
          const float4 zax = za[ix];
          const df zp = two_prod(fx, zax.z);  // table A at (x, c1): zax.x + fx dz, unnormalised
          const df zt = two_sum(zax.x, zp.hi);
          const df gv = df_prop(df{zt.hi, __fadd_rn(zt.lo, __fadd_rn(zax.y, __fmaf_rn(fx, zax.w, zp.lo)))}, x,
                                reg_R_tab(TA, jx, tx, x));
          const float4 zbx = __ldg(zbl + ix);
          const df bp = two_prod(fx, zbx.z);  // table B at (x, c2), unnormalised
          const df bt = two_sum(zbx.x, bp.hi);
          const df g = df_mul_u(gv, df{bt.hi, __fadd_rn(bt.lo, __fadd_rn(zbx.y, __fmaf_rn(fx, zbx.w, bp.lo)))});
          kin.add_prod(df_scale2(rec_w(rp), 2 * m + 1 == n3 ? 1.f : 2.f), g);
        }
        kmid.add_prod(rec_w(r2r), df_mul(kin.sum(), gr1));
      }
      return P.seg[it.seg_off + i * n1 + j] * kmid.value();
    }

    template <int KIND, bool ACC>
    __device__ __forceinline__ double row_value(const RunParams &P, const ItemDev &it, int row, int row0,
                                                const NodeRec *rc, const float *tab, const TableDev *sT,
                                                const int *toff)
    {
      if constexpr (KIND == K_S1) return row_s1<ACC>(P, it, row, rc, tab + toff[0], sT);
      if constexpr (KIND == K_S2) return row_s2<ACC>(P, it, row, rc, tab + toff[0], sT);
      if constexpr (KIND == K_S3) {
        const int sl = it.split_log2;
        return row_s3<ACC>(P, it, row >> sl, row & ((1 << sl) - 1), 1 << sl, rc, tab, sT, toff);
      }
      if constexpr (KIND == K_S3R) {
        const int sl = it.split_log2;
        return row_s3r(P, it, row >> sl, row & ((1 << sl) - 1), 1 << sl, rc, tab, sT, toff);
      }
      if constexpr (KIND == K_S5) return row_s5<ACC>(P, it, row, rc, tab, sT, toff);
      if constexpr (KIND == K_S5Z) {
        const int sl = it.split_log2;
        return narrow_cells(sT[0].a0)
                   ? row_s5z<6>(P, it, row >> sl, row0 >> sl, row & ((1 << sl) - 1), 1 << sl, rc, tab, sT)
                   : row_s5z<9>(P, it, row >> sl, row0 >> sl, row & ((1 << sl) - 1), 1 << sl, rc, tab, sT);
      }
      return 0.0;
    }
  } // namespace

  // resident CTAs per SM the register allocation is held to.  Left to itself the compiler gives
  // S3R 128 registers (16 warps per SM), S2 80 and S5Z 90; these kernels are issue-bound and
  // want the warps: S3R capped at 96 / 80 / 64 registers (128 / 256 / 512 threads) runs 6-8 %
  // faster on C3, S2 at 48 (40 warps per SM, hiding its slice loads) 4 % faster on C2 than at
  // 64, S5Z at 80 gets back the occupancy its earlier form had (measured on GB300; the caps
  // spill a few words at most)
  template <int KIND, int THREADS> constexpr int min_ctas_per_sm()
  {
    if constexpr (KIND == K_S3R) return THREADS == 128 ? 5 : (THREADS == 256 ? 3 : 2);
    if constexpr (KIND == K_S2) return 1280 / THREADS;
    if constexpr (KIND == K_S5Z) return THREADS == 128 ? 6 : (THREADS == 256 ? 3 : 2);
    return 1;
  }

  template <int KIND, bool ACC, int THREADS>
  __global__ void __launch_bounds__(THREADS, (min_ctas_per_sm<KIND, THREADS>()))
      k_fp32c(const RunParams P, int tab_bytes_cap, int rec_cap)
  {
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int NT = Traits<KIND>::kTables;
    // S2, accurate form: the points read the mode-interpolated slices from the segment arena,
    // so only the table's cell-centre reciprocals are staged (the rest of shared memory is
    // left to L1, which holds the slices)
    constexpr bool kRcOnly = KIND == K_S2 && ACC;
    float *tab_s = reinterpret_cast<float *>(smem);
    NodeRec *rec_s0 = reinterpret_cast<NodeRec *>(smem + tab_bytes_cap);
    NodeRec *rec_s1 = rec_s0 + rec_cap;
    __shared__ __align__(8) uint64_t bar[3];
    __shared__ TableDev sT[4];
    __shared__ int s_slot[4], s_toff[4], s_next[2], s_flag, s_tabok;
    __shared__ double red[32];

    if (threadIdx.x == 0) {
      mbar_init(&bar[0], 1);
      mbar_init(&bar[1], 1);
      mbar_init(&bar[2], 1);
      mbar_fence_init();
      for (int i = 0; i < 4; ++i) s_slot[i] = -2;
      s_tabok = 1;
      const int u = P.single ? (int)blockIdx.x : atomicAdd(P.unit_counter, 1);
      s_next[0] = u;
      if (u < P.n_units) issue_records(KIND, P, u, rec_s0, &bar[0]);
    }
    __syncthreads();
    uint32_t ph0 = 0, ph1 = 0, ph_tab = 0;
    int buf = 0;
    for (;;) {
      const int u = s_next[buf];
      if (u >= P.n_units) break;
      const UnitDev U = P.units[u];
      const ItemDev &it = P.items[U.item];
      bool ok = true;
      bool need = false;
#pragma unroll
      for (int t = 0; t < NT; ++t) need |= (it.tab[t] != s_slot[t]);
      if (need) {
        __syncthreads();  // everyone has read s_slot
        if (threadIdx.x == 0) {
          int total = 0;
          for (int t = 0; t < NT; ++t) {
            const int slot = it.tab[t];
            sT[t] = P.tabs[slot];
            s_slot[t] = slot;
            s_toff[t] = total / 4;
            if constexpr (KIND != K_S5Z && KIND != K_S3R) total += kRcOnly ? rc_bytes(sT[t]) : sT[t].bytes;
          }
          // S3R: B's propagator records, then the value records of C and D (table A feeds the
          // hoisted row factors only; B's value records and regulator stay in global memory)
          if constexpr (KIND == K_S3R) {
            bool has = sT[1].gr_off > 0;
            total = 0;
            for (int t = 1; t < 4; ++t) {
              has = has && sT[t].cr_off > 0 && sT[t].n1 == 0;
              s_toff[t] = total / 4;
              total += t == 1 ? s3r_g_bytes(sT[t]) : s3r_rec_bytes(sT[t]);
            }
            if (!has) total = tab_bytes_cap + 1;  // refused below: nothing is staged or evaluated
          }
          // S5Z: table A's cell-centre reciprocals only (both tables share the |q-p|^2 fraction)
          if constexpr (KIND == K_S5Z) total = rc_bytes(sT[0]);
          s_tabok = 1;
          if (total > tab_bytes_cap) {
            atomicOr(P.err, ERR_BAD_INDEX);
            total = 0;
            s_tabok = 0;
          }
          mbar_expect_tx(&bar[2], (uint32_t)total);
          if (total > 0) {
            if constexpr (KIND == K_S5Z) {
              tma_bulk_g2s(tab_s, sT[0].data + sT[0].rc_off, (uint32_t)total, &bar[2]);
            } else if constexpr (KIND == K_S3R) {
              tma_bulk_g2s(tab_s, sT[1].data + sT[1].gr_off, (uint32_t)s3r_g_bytes(sT[1]), &bar[2]);
              for (int t = 2; t < 4; ++t)
                tma_bulk_g2s(tab_s + s_toff[t], sT[t].data + sT[t].cr_off, (uint32_t)s3r_rec_bytes(sT[t]), &bar[2]);
            } else {
              for (int t = 0; t < NT; ++t) {
                if constexpr (kRcOnly) {
                  if (rc_bytes(sT[t]) > 0)
                    tma_bulk_g2s(tab_s + s_toff[t], sT[t].data + sT[t].rc_off, (uint32_t)rc_bytes(sT[t]), &bar[2]);
                } else
                  tma_bulk_g2s(tab_s + s_toff[t], sT[t].data, (uint32_t)sT[t].bytes, &bar[2]);
              }
            }
          }
        }
        __syncthreads();
        ok = mbar_wait_bounded(&bar[2], ph_tab, P.err) && ok;
        ph_tab ^= 1;
      }
      if (!s_tabok) {
        ok = false;  // the tables of this unit could not be staged (error word set)
      }
      // prefetch the next unit's records into the other buffer
      if (threadIdx.x == 0) {
        const int un = P.single ? P.n_units : atomicAdd(P.unit_counter, 1);
        s_next[buf ^ 1] = un;
        if (un < P.n_units) issue_records(KIND, P, un, buf ? rec_s0 : rec_s1, &bar[buf ^ 1]);
      }
      if (buf == 0) {
        ok = mbar_wait_bounded(&bar[0], ph0, P.err) && ok;
        ph0 ^= 1;
      } else {
        ok = mbar_wait_bounded(&bar[1], ph1, P.err) && ok;
        ph1 ^= 1;
      }
      // a unit holds rows_per_thread x THREADS rows (the schedule's choice); thread t takes rows
      // t, t + THREADS, ...
      double acc = 0.0;
      if (ok) {
#pragma unroll 1
        for (int r = threadIdx.x; r < U.row_count; r += THREADS)
          acc += row_value<KIND, ACC>(P, it, U.row_begin + r, U.row_begin, buf ? rec_s1 : rec_s0, tab_s, sT,
                                      s_toff);
      }
      const double tot = block_sum(acc, red);
      unit_finish(P, U.slot, U.item, tot, red, &s_flag);
      buf ^= 1;
    }
  }

  // ------------------------------------------------------------------------------------------
  // launch plumbing
  // ------------------------------------------------------------------------------------------
  namespace
  {
    template <int KIND, bool ACC, int THREADS> const void *kfun() { return (const void *)&k_fp32c<KIND, ACC, THREADS>; }

    template <int KIND, bool ACC> const void *sel_threads(int threads)
    {
      if (threads == 128) return kfun<KIND, ACC, 128>();
      if (threads == 256) return kfun<KIND, ACC, 256>();
      if (threads == 512) return kfun<KIND, ACC, 512>();
      return nullptr;
    }

    const void *select(int kind, int threads)
    {
      const bool acc = kind_acc(kind);
      switch (kind_base(kind)) {
      case K_S1:
        return acc ? sel_threads<K_S1, true>(threads) : sel_threads<K_S1, false>(threads);
      case K_S2:
        return acc ? sel_threads<K_S2, true>(threads) : sel_threads<K_S2, false>(threads);
      case K_S3:
        return acc ? sel_threads<K_S3, true>(threads) : sel_threads<K_S3, false>(threads);
      case K_S5:
        return acc ? sel_threads<K_S5, true>(threads) : sel_threads<K_S5, false>(threads);
      case K_S5Z:
        return acc ? sel_threads<K_S5Z, true>(threads) : nullptr;
      case K_S3R:
        return acc ? sel_threads<K_S3R, true>(threads) : nullptr;
      }
      return nullptr;
    }
  } // namespace

  int kind_default_threads(int kind) { return kind_default_schedule(kind).threads; }

  // defaults measured on GB300 (the autotuner's landscapes on the benchmark workloads): S5Z runs
  // 23 % faster at 256 threads with its c2 loop split over two threads than at 512 unsplit; S3R
  // 5 % faster at 256 threads (80 registers, 3 CTAs per SM) than at 128 (96, 5 CTAs)
  gb_schedule kind_default_schedule(int kind)
  {
    switch (kind_base(kind)) {
    case K_S1:
      return gb_schedule{128, 1, 1, GB_ORDER_ITEM};
    case K_S5:
      return gb_schedule{512, 1, 1, GB_ORDER_ITEM};
    case K_S5Z:
      return gb_schedule{256, 1, 2, GB_ORDER_ITEM};
    case K_S3R:
      return gb_schedule{256, 2, 1, GB_ORDER_ITEM};
    default:
      return gb_schedule{256, 1, 1, GB_ORDER_ITEM};
    }
  }

  // the kernels' dynamic shared-memory limit is raised once per (kernel, device) to the largest
  // size launched so far, instead of a driver call on every launch
  static cudaError_t ensure_max_smem(const void *fn, size_t smem)
  {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, size_t> set;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    size_t &have = set[{fn, dev}];
    if (smem <= have) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) have = smem;
    return e;
  }

  cudaError_t launch_fp32c(int kind, const RunParams &P, int threads, int ctas, int tab_bytes_cap, int rec_cap,
                           cudaStream_t s)
  {
    const void *fn = select(kind, threads);
    if (!fn) return cudaErrorInvalidValue;
    const size_t smem = (size_t)tab_bytes_cap + 2 * (size_t)rec_cap * sizeof(NodeRec);
    cudaError_t e = ensure_max_smem(fn, smem);
    if (e != cudaSuccess) return e;
    RunParams p = P;
    void *args[] = {(void *)&p, (void *)&tab_bytes_cap, (void *)&rec_cap};
    return cudaLaunchKernel(fn, dim3(ctas), dim3(threads), args, smem, s);
  }

  int fp32c_occupancy(int kind, int threads, int tab_bytes_cap, int rec_cap)
  {
    const void *fn = select(kind, threads);
    if (!fn) return 0;
    const size_t smem = (size_t)tab_bytes_cap + 2 * (size_t)rec_cap * sizeof(NodeRec);
    if (ensure_max_smem(fn, smem) != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess) return 0;
    return nb;
  }
} // namespace gbint
