// integrands.hh -- TEST INFRASTRUCTURE ONLY (see oracle.hh).
//
// FP64 definitions of the integrand catalogue.  The CUDA engine evaluates the same
// functions (diffrg_gb300/csrc/integrands.cuh); every definition here is the checker's copy.
//
//   id 0  POLY   product of polynomials in each coordinate, the KERNEL of the reference's
//                integrator tests (e.g. DiFfRG/tests/physics/integration/integrator_4D_gpu.cu:14-39)
//   id 1  PROP1  sqrt(1-c^2) G(q^2) G(q^2+p^2+2pqc) Rdot(q^2) * kfac     (d=4 propagator loop)
//   id 3  PROP3  Rdot(q^2) G_A(q^2) G_B(|q-p|^2) V_C(s) V_D(|q-p/2|^2)   (3D four-table loop)
//   id 5  VERT4  Rdot(q^2) G(q^2,c1) G(|q-p1|^2,c2) G(|q+p2|^2,c1) V(|q+p2|^2,c2) (4D vertex)
//   W2           finite-T loop q^2 G(w,q^2) G(w,|q+p|^2) Rdot(q^2) summed over Matsubara modes
//
// G(x) = 1/(Z(x) x + R(x)) with R the b=1 bosonic regulator at k=1 (regulators.hh:76-79).
#pragma once

#include "families.hh"

namespace oracle
{
  enum Integrand : int { IG_POLY = 0, IG_PROP1 = 1, IG_PROP3 = 3, IG_VERT4 = 5 };

  constexpr int kArgs = 24;  // per-integral argument slots

  struct Tables {
    Table t[4];
  };

  inline double G1(const Table &Z, double x)
  {
    return 1.0 / (Z(x) * x + reg_RB(1.0, x));
  }
  inline double G2d(const Table &Z, double x, double t)
  {
    return 1.0 / (Z(x, t) * x + reg_RB(1.0, x));
  }

  inline double poly(const double *c, int n, double x)
  {
    double r = 0;
    for (int i = n - 1; i >= 0; --i) r = r * x + c[i];
    return r;
  }

  // POLY argument layout: [c, q0..q5, a1_0..3, a2_0..3, a3_0..3, t0..3, mode]; the q0 factor is
  // the cubic t(q0), or 1/t(q0) when mode != 0 (the finite-T tests of the reference divide by a
  // polynomial in q0, DiFfRG/tests/physics/integration_finiteT/integrator_4D_finiteTq0_gpu.cu:19-28)
  inline double poly_q0(const double *a, double q0)
  {
    const double v = poly(a + 19, 4, q0);
    return a[23] != 0 ? 1.0 / v : v;
  }
  inline double poly_kernel(int family, const Point &P, const double *a)
  {
    const double *pq = a + 1, *p1 = a + 7, *p2 = a + 11, *p3 = a + 15;
    switch (family) {
    case F_1D:
      return poly(pq, 6, P.q);
    case F_ANGLE:
      return poly(pq, 6, P.q) * poly(p1, 4, P.c1);
    case F_3D:
      return poly(pq, 6, P.q) * poly(p1, 4, P.c1) * poly(p2, 4, P.phi);
    case F_4D2ANG:
      return poly(pq, 6, P.q) * poly(p1, 4, P.c1) * poly(p2, 4, P.c2);
    case F_4D:
      return poly(pq, 6, P.q) * poly(p1, 4, P.c1) * poly(p2, 4, P.c2) * poly(p3, 4, P.phi);
    case F_CART1:
      return poly(pq, 6, P.qx);
    case F_CART2:
      return poly(pq, 6, P.qx) * poly(p1, 4, P.qy);
    case F_CART3:
      return poly(pq, 6, P.qx) * poly(p1, 4, P.qy) * poly(p2, 4, P.qz);
    case F_2DPQ0:
    case F_2DPX0:
    case F_ANGLE_FTQ0:
    case F_ANGLE_FTX0:
      return poly(pq, 6, P.q) * poly(p1, 4, P.c1) * poly_q0(a, P.q0);
    case F_3DPQ0:
    case F_3DPX0:
    case F_4D_FTQ0:
    case F_4D_FTX0:
      return poly(pq, 6, P.q) * poly(p1, 4, P.c1) * poly(p2, 4, P.phi) * poly_q0(a, P.q0);
    case F_FTQ0:
    case F_FTX0:
      return poly(pq, 6, P.q) * poly_q0(a, P.q0);
    case F_CONST:
      return poly(pq, 6, P.k);
    }
    return 0;
  }

  // PROP1 args: [c, p, kfac]
  inline double prop1_kernel(const Tables &T, const Point &P, const double *a)
  {
    const double p = a[1], q = P.q, c = P.c1;
    const double q2 = q * q;
    double x2 = q2 + p * p + 2 * p * q * c;
    if (x2 < 1e-300) x2 = 1e-300;
    return a[2] * std::sqrt(1 - c * c) * G1(T.t[0], q2) * G1(T.t[0], x2) * reg_RBdot(1.0, q2);
  }

  // PROP3 args: [c, P, cos(theta_p), sin(theta_p)]
  inline double prop3_kernel(const Tables &T, const Point &P, const double *a)
  {
    const double p = a[1], ct = a[2], st = a[3];
    const double q = P.q, c = P.c1, s = std::sqrt(1 - c * c), cf = std::cos(P.phi);
    const double q2 = q * q;
    const double qp = q * p * (c * ct + s * st * cf);
    double r2 = q2 + p * p - 2 * qp;
    double t2 = q2 + 0.25 * p * p - qp;
    if (r2 < 1e-300) r2 = 1e-300;
    if (t2 < 1e-300) t2 = 1e-300;
    const double sv = (q2 + r2 + p * p) / 3.0;
    return reg_RBdot(1.0, q2) * G1(T.t[0], q2) * G1(T.t[1], r2) * T.t[2](sv) * T.t[3](t2);
  }

  // VERT4 args: [c, P, cos(alpha), sin(alpha)];  p1 = P(1,0,0,0), p2 = P(cos a, 0, sin a, 0),
  // q = q (c1, s1 c2, s1 s2 cos phi, s1 s2 sin phi)
  inline double vert4_kernel(const Tables &T, const Point &P, const double *a)
  {
    const double p = a[1], ca = a[2], sa = a[3];
    const double q = P.q, c1 = P.c1, c2 = P.c2;
    const double s1 = std::sqrt(1 - c1 * c1), s2 = std::sqrt(1 - c2 * c2);
    const double q2 = q * q, pp = p * p;
    double r1 = q2 + pp - 2 * q * p * c1;
    double r2 = q2 + pp + 2 * q * p * (c1 * ca + s1 * s2 * std::cos(P.phi) * sa);
    if (r1 < 1e-300) r1 = 1e-300;
    if (r2 < 1e-300) r2 = 1e-300;
    return reg_RBdot(1.0, q2) * G2d(T.t[0], q2, c1) * G2d(T.t[0], r1, c2) * G2d(T.t[0], r2, c1) *
           T.t[1](r2, c2);
  }

  inline double eval_kernel(int integrand, int family, const Tables &T, const Point &P, const double *a)
  {
    switch (integrand) {
    case IG_POLY:
      return poly_kernel(family, P, a);
    case IG_PROP1:
      return prop1_kernel(T, P, a);
    case IG_PROP3:
      return prop3_kernel(T, P, a);
    case IG_VERT4:
      return vert4_kernel(T, P, a);
    }
    throw std::invalid_argument("unknown integrand");
  }

  // ---------------------------------------------------------------------------------------
  // Direct workload sums with radial Gauss-Legendre in q (not x = q^2/k^2)
  // ---------------------------------------------------------------------------------------

  // W1: (4 pi / (2 pi)^4) int_0^qmax dq int_-1^1 dc  q^3 sqrt(1-c^2) G(q^2) G(q^2+p^2+2pqc) Rdot(q^2)
  inline double w1(const Tables &T, int nq, int nc, double qmax, double p)
  {
    const auto &Q = rules().get(nq);
    const auto &C = rules().get(nc);
    const double pref = 4 * kPi / powi(2 * kPi, 4);
    PairwiseSum acc;
    for (int i = 0; i < nq; ++i) {
      const double q = qmax * Q.first[i], wq = qmax * Q.second[i];
      const double q2 = q * q;
      const double outer = q2 * q * G1(T.t[0], q2) * reg_RBdot(1.0, q2);
      for (int l = 0; l < nc; ++l) {
        const double c = 2 * C.first[l] - 1, wc = 2 * C.second[l];
        double x2 = q2 + p * p + 2 * p * q * c;
        if (x2 < 1e-300) x2 = 1e-300;
        acc.add(pref * wq * wc * outer * std::sqrt(1 - c * c) * G1(T.t[0], x2));
      }
    }
    return acc.total();
  }

  // W2: finite-T 3+1D loop, explicit bosonic sum n = -M..M at omega_n = 2 pi T n, external
  // frequency W (0 in the benchmark):
  //   T sum_n (2 pi / (2 pi)^3) int_0^qmax dq int dc q^2 G(w_n,q^2) G(w_n+W,q^2+p^2+2pqc) Rdot(q^2)
  //   G(w,x) = 1/(Z(|w|/(2 pi T), sqrt x) (w^2 + x) + R(x)),  Z a 2D table (mode index, |q|)
  inline double w2_G(const Table &Z, double w, double x, double T)
  {
    const double nidx = std::fabs(w) / (2 * kPi * T);
    return 1.0 / (Z(nidx, std::sqrt(x)) * (w * w + x) + reg_RB(1.0, x));
  }
  inline double w2(const Tables &Tb, int M, int nq, int nc, double qmax, double p, double T, double Om = 0.0)
  {
    const auto &Q = rules().get(nq);
    const auto &C = rules().get(nc);
    const double pref = T * 2 * kPi / powi(2 * kPi, 3);
    PairwiseSum acc;
    for (int m = 0; m <= M; ++m) {
      const double w = 2 * kPi * T * m;
      for (int i = 0; i < nq; ++i) {
        const double q = qmax * Q.first[i], wq = qmax * Q.second[i];
        const double q2 = q * q;
        const double rd = reg_RBdot(1.0, q2);
        for (int l = 0; l < nc; ++l) {
          const double c = 2 * C.first[l] - 1, wc = 2 * C.second[l];
          double x2 = q2 + p * p + 2 * p * q * c;
          if (x2 < 1e-300) x2 = 1e-300;
          double v = q2 * rd * w2_G(Tb.t[0], w, q2, T) * w2_G(Tb.t[0], w + Om, x2, T);
          if (m > 0) v += q2 * rd * w2_G(Tb.t[0], -w, q2, T) * w2_G(Tb.t[0], -w + Om, x2, T);
          acc.add(pref * wq * wc * v);
        }
      }
    }
    return acc.total();
  }
} // namespace oracle
