// integrands.cuh -- the compiled-in integrand catalogue (device code).
//
// FP64 forms are evaluated point by point by the generic kernel and the reference-pattern
// path; the FP32-compensated kernels (kernels_fp32c.cu) evaluate the same functions with
// their one-axis factors hoisted to FP64.  Definitions:
//   POLY   prod of polynomials per coordinate -- the PolyIntegrand KERNEL of the reference
//          integrator tests (DiFfRG/tests/physics/integration/integrator_4D_gpu.cu:14-39)
//   PROP1  kfac sqrt(1-c^2) G(q^2) G(q^2+p^2+2pqc) Rdot(q^2)              args [c, p, kfac]
//   PROP3  Rdot(q^2) G_A(q^2) G_B(r^2) V_C(s) V_D(t^2), r = |q-p|, t = |q-p/2|,
//          s = (q^2+r^2+p^2)/3, p at polar angle theta_p     args [c, P, cos th_p, sin th_p]
//   VERT4  Rdot(q^2) G(q^2,c1) G(r1^2,c2) G(r2^2,c1) V(r2^2,c2), r1 = |q-p1|, r2 = |q+p2|,
//          p1 = P(1,0,0,0), p2 = P(cos a,0,sin a,0)            args [c, P, cos a, sin a]
//   FTLOOP G(w,q^2) G(w+W,q^2+p^2+2pqc) Rdot(q^2), G(w,x) = 1/(Z(|w|/(2 pi T), sqrt x)(w^2+x)+R(x)),
//          W the external frequency                             args [c, p, T, W]
// with G(x) = 1/(Z(x) x + R(x)), R the b=1 bosonic regulator (regulators.hh:76-99) at k = 1.
#pragma once

#include "engine_types.hh"

namespace gbint
{
  namespace dev
  {
    struct Pt {
      double q, c1, c2, phi, q0, qx, qy, qz, k;
    };

    __device__ __forceinline__ double tab1_64(const TableDev &t, double x)
    {
      int i;
      const double f = axis_frac64(t.a0, x, i);
      return lerp64((double)t.data[i], (double)t.data[i + 1], f);
    }
    __device__ __forceinline__ double tab2_64(const TableDev &t, double x, double y)
    {
      int i, j;
      const double fx = axis_frac64(t.a0, x, i);
      const double fy = axis_frac64(t.a1, y, j);
      const float *d = t.data;
      const int n1 = t.n1;
      const double lo = lerp64((double)d[i * n1 + j], (double)d[(i + 1) * n1 + j], fx);
      const double hi = lerp64((double)d[i * n1 + j + 1], (double)d[(i + 1) * n1 + j + 1], fx);
      return lerp64(lo, hi, fy);
    }
    __device__ __forceinline__ double G1_64(const TableDev &t, double x) { return 1.0 / (tab1_64(t, x) * x + reg_R(x)); }
    __device__ __forceinline__ double G2_64(const TableDev &t, double x, double y)
    {
      return 1.0 / (tab2_64(t, x, y) * x + reg_R(x));
    }

    __device__ __forceinline__ double poly64(const double *c, int n, double x)
    {
      double r = 0;
      for (int i = n - 1; i >= 0; --i) r = r * x + c[i];
      return r;
    }

    // POLY args: [c, q0..q5, a1_0..3, a2_0..3, a3_0..3, t0..3, mode]; q0 factor t(q0), or 1/t(q0)
    // for mode != 0 (the finite-T test kernels divide by a polynomial in q0)
    __device__ __forceinline__ double poly_q0(const double *a, double q0)
    {
      const double v = poly64(a + 19, 4, q0);
      return a[23] != 0.0 ? 1.0 / v : v;
    }
    __device__ inline double ig_poly(int family, const Pt &P, const double *a)
    {
      const double *pq = a + 1, *p1 = a + 7, *p2 = a + 11, *p3 = a + 15;
      switch (family) {
      case GB_FAM_1D:
        return poly64(pq, 6, P.q);
      case GB_FAM_ANGLE:
      case GB_FAM_QLOOP:
        return poly64(pq, 6, P.q) * poly64(p1, 4, P.c1);
      case GB_FAM_3D:
        return poly64(pq, 6, P.q) * poly64(p1, 4, P.c1) * poly64(p2, 4, P.phi);
      case GB_FAM_4D2ANG:
        return poly64(pq, 6, P.q) * poly64(p1, 4, P.c1) * poly64(p2, 4, P.c2);
      case GB_FAM_4D:
        return poly64(pq, 6, P.q) * poly64(p1, 4, P.c1) * poly64(p2, 4, P.c2) * poly64(p3, 4, P.phi);
      case GB_FAM_CART1:
        return poly64(pq, 6, P.qx);
      case GB_FAM_CART2:
        return poly64(pq, 6, P.qx) * poly64(p1, 4, P.qy);
      case GB_FAM_CART3:
        return poly64(pq, 6, P.qx) * poly64(p1, 4, P.qy) * poly64(p2, 4, P.qz);
      case GB_FAM_2DPQ0:
      case GB_FAM_2DPX0:
      case GB_FAM_ANGLE_FTQ0:
      case GB_FAM_ANGLE_FTX0:
      case GB_FAM_QLOOP_T:
        return poly64(pq, 6, P.q) * poly64(p1, 4, P.c1) * poly_q0(a, P.q0);
      case GB_FAM_3DPQ0:
      case GB_FAM_3DPX0:
      case GB_FAM_4D_FTQ0:
      case GB_FAM_4D_FTX0:
        return poly64(pq, 6, P.q) * poly64(p1, 4, P.c1) * poly64(p2, 4, P.phi) * poly_q0(a, P.q0);
      case GB_FAM_FTQ0:
      case GB_FAM_FTX0:
        return poly64(pq, 6, P.q) * poly_q0(a, P.q0);
      case GB_FAM_CONST:
        return poly64(pq, 6, P.k);
      }
      return 0.0;
    }

    __device__ inline double ig_prop1(const Pt &P, const double *a, const TableDev *T)
    {
      const double p = a[1], q = P.q, c = P.c1, q2 = q * q;
      double x2 = q2 + p * p + 2 * p * q * c;
      x2 = fmax(x2, 1e-300);
      return a[2] * sqrt(1 - c * c) * G1_64(T[0], q2) * G1_64(T[0], x2) * reg_Rdot(q2);
    }

    __device__ inline double ig_prop3(const Pt &P, const double *a, const TableDev *T)
    {
      const double p = a[1], ct = a[2], st = a[3];
      const double q = P.q, c = P.c1, s = sqrt(1 - c * c), cf = cos(P.phi);
      const double q2 = q * q;
      const double qp = q * p * (c * ct + s * st * cf);
      const double r2 = fmax(q2 + p * p - 2 * qp, 1e-300);
      const double t2 = fmax(q2 + 0.25 * p * p - qp, 1e-300);
      const double sv = (q2 + r2 + p * p) / 3.0;
      return reg_Rdot(q2) * G1_64(T[0], q2) * G1_64(T[1], r2) * tab1_64(T[2], sv) * tab1_64(T[3], t2);
    }

    __device__ inline double ig_vert4(const Pt &P, const double *a, const TableDev *T)
    {
      const double p = a[1], ca = a[2], sa = a[3];
      const double q = P.q, c1 = P.c1, c2 = P.c2;
      const double s1 = sqrt(1 - c1 * c1), s2 = sqrt(1 - c2 * c2);
      const double q2 = q * q, pp = p * p;
      const double r1 = fmax(q2 + pp - 2 * q * p * c1, 1e-300);
      const double r2 = fmax(q2 + pp + 2 * q * p * (c1 * ca + s1 * s2 * cos(P.phi) * sa), 1e-300);
      return reg_Rdot(q2) * G2_64(T[0], q2, c1) * G2_64(T[0], r1, c2) * G2_64(T[0], r2, c1) * tab2_64(T[1], r2, c2);
    }

    __device__ __forceinline__ double ft_G64(const TableDev &Z, double w, double x, double T)
    {
      const double nidx = fabs(w) / (2 * 3.14159265358979323846 * T);
      return 1.0 / (tab2_64(Z, nidx, sqrt(x)) * (w * w + x) + reg_R(x));
    }
    __device__ inline double ig_ftloop(const Pt &P, const double *a, const TableDev *T)
    {
      const double p = a[1], Tt = a[2], Om = a[3], q = P.q, c = P.c1, q2 = q * q;
      const double x2 = fmax(q2 + p * p + 2 * p * q * c, 1e-300);
      return reg_Rdot(q2) * ft_G64(T[0], P.q0, q2, Tt) * ft_G64(T[0], P.q0 + Om, x2, Tt);
    }

    __device__ __forceinline__ double ig_eval64(int ig, int family, const Pt &P, const double *a, const TableDev *T)
    {
      switch (ig) {
      case GB_IG_POLY:
        return ig_poly(family, P, a);
      case GB_IG_PROP1:
        return ig_prop1(P, a, T);
      case GB_IG_PROP3:
        return ig_prop3(P, a, T);
      case GB_IG_VERT4:
        return ig_vert4(P, a, T);
      case GB_IG_FTLOOP:
        return ig_ftloop(P, a, T);
      }
      return 0.0;
    }

    __device__ __forceinline__ void set_role(Pt &P, int role, double v)
    {
      switch (role) {
      case R_Q: P.q = v; break;
      case R_C1: P.c1 = v; break;
      case R_C2: P.c2 = v; break;
      case R_PHI: P.phi = v; break;
      case R_Q0: P.q0 = v; break;
      case R_QX: P.qx = v; break;
      case R_QY: P.qy = v; break;
      case R_QZ: P.qz = v; break;
      default: break;
      }
    }

    // One grid point of an FP64 item: the flattened index `pt` is split into one node per axis
    // (last axis fastest), the node values set the integrand's coordinates and the node weights
    // multiply; axes with +-q0 pairs add the integrand at -q0 from node pm_from on.  The one
    // definition behind every FP64 kernel that walks an item's grid (k_generic, k_generic_noalloc),
    // so their results agree bit for bit.
    __device__ __forceinline__ double eval_point_fp64(const ItemDev &it, long long pt, const double *pv,
                                                      const double *pw, const TableDev *T)
    {
      Pt P{0, 0, 0, 0, 0, 0, 0, 0, it.k};
      double w = 1.0;
      bool pm = false;
      long long rem = pt;
      for (int a = it.n_axes - 1; a >= 0; --a) {
        const AxisRef ax = it.ax[a];
        const int idx = (int)(rem % ax.n);
        rem /= ax.n;
        const int node = ax.off + idx;
        set_role(P, ax.role, pv[node]);
        w *= pw[node];
        if (idx >= ax.pm_from) pm = true;
      }
      double f = ig_eval64(it.integrand, it.family, P, it.args, T);
      if (pm) {
        P.q0 = -P.q0;
        f += ig_eval64(it.integrand, it.family, P, it.args, T);
      }
      return w * f;
    }
  } // namespace dev
} // namespace gbint
