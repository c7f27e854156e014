// regulators.hh -- FRG regulator shape functions for user KERNELs, without dependencies.
//
// The classes of DiFfRG/include/DiFfRG/physics/regulators.hh with the same names, options
// structs and static functions (host and device, any arithmetic or gbint::dual result type):
//   LitimRegulator                 R_B = (k^2 - q^2) theta(k^2 - q^2)                   (:24-51)
//   BosonicRegulator<Opts{b}>      R_B = q^2 x^(b-1) / (e^(x^b) - 1),  x = q^2/k^2       (:72-123)
//   ExponentialRegulator<Opts{b}>  R_B = k^2 e^(-x^b)                                   (:144-191)
//   SmoothedLitimRegulator<Opts{alpha}>
//                                  R_B = (k^2 - q^2) / (1 + e^((x - 1)/alpha))          (:212-242)
//   PolynomialExpRegulator<Opts{order}>
//                                  R_B = k^2 e^(-f(x)),  f(x) = sum_{n=1..order} x^n/n  (:625-695)
// Functions (as in the reference): RB = R_B(k^2, q^2); RBdot = d/dt R_B with t = ln k;
// dq2RB = dR_B/dq^2; RF = sqrt(R_B + q^2) - sqrt(q^2) (fermionic, p r_F); RFdot = dRF/dt;
// dq2RF = dRF/dq^2.  The derivatives are written out from the shapes above.
//   RationalExpRegulator<Opts{order, c, b0}>
//                                  R_B = k^2 e^(-f(x)),  f = P/D rational              (:244-600)
// RationalExpRegulator's f is built here from its defining properties rather than from the
// reference's per-order expressions: D(x) = 1 + b0 x^m + g x^(n-1) (n = order, m = floor(n/2),
// g = a/(c-1), a = 1/n + b0/ceil(n/2)) and P = the part of degree <= n of D(x) L(x), with
// L(x) = sum_{i>=1} x^i/i = -ln(1-x).  So f = -ln(1-x) + O(x^n) near 0 (R_B = k^2(1 - x) + ...,
// a pole of order n in the propagator once the mass turns negative) and f -> c x for large x
// (tail e^(-c x)); P and D reproduce the reference's expressions for every order 1..16.
#pragma once

#include <cmath>
#include <type_traits>
#include <utility>

#ifndef GBINT_REG_HD
#define GBINT_REG_HD __host__ __device__ __forceinline__
#endif

namespace DiFfRG
{
  namespace gbint_reg
  {
    // x^e for a compile-time exponent: repeated products when e is integral, pow otherwise
    template <typename T, typename E> GBINT_REG_HD T ipow(T x, E e)
    {
      using std::pow;
      const int n = (int)e;
      if ((E)n == e && n >= 0 && n <= 16) {
        T r = T(1);
        for (int i = 0; i < n; ++i) r = r * x;
        return r;
      }
      return pow(x, e);
    }
  } // namespace gbint_reg

  template <class Dummy = void> struct LitimRegulator {
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RB(const NT1 k2, const NT2 q2)
    {
      return (k2 - q2) * (k2 > q2);
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RBdot(const NT1 k2, const NT2 q2)
    {
      return 2. * k2 * (k2 > q2);
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RF(const NT1 k2, const NT2 q2)
    {
      using std::sqrt;
      return sqrt(RB(k2, q2) + q2) - sqrt(q2);
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RFdot(const NT1 k2, const NT2 q2)
    {
      using std::sqrt;
      return 0.5 * RBdot(k2, q2) / sqrt(RB(k2, q2) + q2);
    }
    // not differentiable at q^2 = k^2 (as in the reference, a call does not compile)
    template <typename NT1, typename NT2> static void dq2RB(const NT1, const NT2) = delete;
  };

  // the fermionic functions and dq2RF of a bosonic shape RB, RBdot, dq2RB
  template <class R> struct FermionicFromBosonic {
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RF(const NT1 k2, const NT2 q2)
    {
      using std::sqrt;
      return sqrt(R::RB(k2, q2) + q2) - sqrt(q2);
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RFdot(const NT1 k2, const NT2 q2)
    {
      using std::sqrt;
      return 0.5 * R::RBdot(k2, q2) / sqrt(R::RB(k2, q2) + q2);
    }
    // d/dq^2 [sqrt(RB + q^2) - q] = (1 + dq2RB) / (2 sqrt(RB + q^2)) - 1 / (2 q)
    template <typename NT1, typename NT2> static GBINT_REG_HD auto dq2RF(const NT1 k2, const NT2 q2)
    {
      using std::sqrt;
      const auto q = sqrt(q2);
      return (-1. + q * (1. + R::dq2RB(k2, q2)) / (q + RF(k2, q2))) / (2. * q);
    }
  };

  struct BosonicRegulatorOpts {
    static constexpr double b = 2.;
  };
  template <class OPTS = BosonicRegulatorOpts>
  struct BosonicRegulator : FermionicFromBosonic<BosonicRegulator<OPTS>> {
    static constexpr double b = OPTS::b;
    // R = q^2 x^(b-1) / (e^(x^b) - 1) = k^2 x^b / expm1(x^b)
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RB(const NT1 k2, const NT2 q2)
    {
      using std::expm1;
      const auto x = q2 / k2;
      return q2 * gbint_reg::ipow(x, b - 1.) / expm1(gbint_reg::ipow(x, b));
    }
    // dR/dq^2 = d/dx [x^b / expm1(x^b)] = b x^(b-1) (expm1(y) - y e^y) / expm1(y)^2, y = x^b
    template <typename NT1, typename NT2> static GBINT_REG_HD auto dq2RB(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      using std::expm1;
      const auto x = q2 / k2;
      const auto y = gbint_reg::ipow(x, b);
      const auto em = expm1(y);
      return b * gbint_reg::ipow(x, b - 1.) * (em - y * exp(y)) / (em * em);
    }
    // d/dt at fixed q^2 (dx/dt = -2x): 2 k^2 y (expm1(y) (1 - b) + b y e^y) / expm1(y)^2
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RBdot(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      using std::expm1;
      const auto y = gbint_reg::ipow(q2 / k2, b);
      const auto em = expm1(y);
      return 2. * k2 * y * (em * (1. - b) + b * y * exp(y)) / (em * em);
    }
  };

  struct ExponentialRegulatorOpts {
    static constexpr double b = 2.;
  };
  template <class OPTS = ExponentialRegulatorOpts>
  struct ExponentialRegulator : FermionicFromBosonic<ExponentialRegulator<OPTS>> {
    static constexpr double b = OPTS::b;
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RB(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      return k2 * exp(-gbint_reg::ipow(q2 / k2, b));
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto dq2RB(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      const auto x = q2 / k2;
      const auto xm = gbint_reg::ipow(x, b - 1.);
      return -b * xm * exp(-xm * x);
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RBdot(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      const auto y = gbint_reg::ipow(q2 / k2, b);
      return 2. * k2 * exp(-y) * (1. + b * y);
    }
  };

  struct SmoothedLitimRegulatorOpts {
    static constexpr double alpha = 2e-3;
  };
  template <class OPTS = SmoothedLitimRegulatorOpts> struct SmoothedLitimRegulator {
    static constexpr double alpha = OPTS::alpha;
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RB(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      return (k2 - q2) / (1. + exp((q2 / k2 - 1.) / alpha));
    }
    // d/dt, x = q^2/k^2, E = e^((x-1)/alpha): 2 k^2 (1 + E (x - x^2 + alpha) / alpha) / (1 + E)^2
    // (0 where E overflows the numerator: R and its derivative vanish there)
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RBdot(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      const auto x = q2 / k2;
      const auto E = exp((x - 1.) / alpha);
      const auto d = 2. * k2 * (1. + E * (x - x * x + alpha) / alpha) / ((1. + E) * (1. + E));
      return E > 1e50 ? decltype(d)(0.) : d;
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RF(const NT1 k2, const NT2 q2)
    {
      using std::sqrt;
      return sqrt(RB(k2, q2) + q2) - sqrt(q2);
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RFdot(const NT1 k2, const NT2 q2)
    {
      using std::sqrt;
      return 0.5 * RBdot(k2, q2) / sqrt(RB(k2, q2) + q2);
    }
  };

  struct PolynomialExpRegulatorOpts {
    static constexpr int order = 8;
  };
  template <class OPTS = PolynomialExpRegulatorOpts>
  struct PolynomialExpRegulator : FermionicFromBosonic<PolynomialExpRegulator<OPTS>> {
    static constexpr int order = OPTS::order;
    static_assert(order > 0, "PolynomialExpRegulator: order must be > 0");
    // f(x) = sum_{n=1..order} x^n / n and f'(x) = sum_{n=0..order-1} x^n, by Horner
    template <typename T> static GBINT_REG_HD T f(T x)
    {
      T r = T(1.0 / order);
      for (int n = order - 1; n >= 1; --n) r = r * x + T(1.0 / n);
      return r * x;
    }
    template <typename T> static GBINT_REG_HD T df(T x)
    {
      T r = T(1);
      for (int n = order - 2; n >= 0; --n) r = r * x + T(1);
      return r;
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RB(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      const auto x = q2 / k2;
      return k2 * exp(-f(x));
    }
    // d/dt at fixed q^2: 2 k^2 e^(-f) (1 + x f'(x))
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RBdot(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      const auto x = q2 / k2;
      return 2. * k2 * exp(-f(x)) * (1. + df(x) * x);
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto dq2RB(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      const auto x = q2 / k2;
      return -exp(-f(x)) * df(x);
    }
  };

  struct RationalExpRegulatorOpts {
    static constexpr int order = 8;
    constexpr static double c = 2;
    constexpr static double b0 = 0.;
  };
  template <class OPTS = RationalExpRegulatorOpts>
  struct RationalExpRegulator : FermionicFromBosonic<RationalExpRegulator<OPTS>> {
    static constexpr int order = OPTS::order;
    static_assert(order > 0, "RationalExpRegulator: order must be positive");
    constexpr static double c = OPTS::c;
    constexpr static double b0 = OPTS::b0;
    static_assert(c != 1.0, "RationalExpRegulator: c = 1 has no tail");

    // coefficients of D (degree order-1) and P (degree order, no constant term); constant-evaluated
    static constexpr int m_ = order / 2;
    static constexpr double g_ = (1.0 / order + b0 / (order - m_)) / (c - 1.0);
    static constexpr double dcoef(int l)
    {
      return (l == 0 ? 1.0 : 0.0) + (l == m_ ? b0 : 0.0) + (l == order - 1 ? g_ : 0.0);
    }
    static constexpr double pcoef(int i)  // [x^i] (D L), i = 1..order
    {
      double s = 0.0;
      for (int l = 0; l < i && l < order; ++l) s += dcoef(l) / (double)(i - l);
      return s;
    }

    // Horner sums with compile-time coefficients: sum_{i=I..N} C(i) x^(i-I)
    template <int I, typename T> static GBINT_REG_HD T hornerP(const T &x)  // P(x)/x
    {
      constexpr double cf = pcoef(I);
      if constexpr (I == order)
        return T(cf);
      else
        return hornerP<I + 1>(x) * x + T(cf);
    }
    template <int I, typename T> static GBINT_REG_HD T hornerdP(const T &x)  // P'(x)
    {
      constexpr double cf = I * pcoef(I);
      if constexpr (I == order)
        return T(cf);
      else
        return hornerdP<I + 1>(x) * x + T(cf);
    }
    template <int I, typename T> static GBINT_REG_HD T hornerD(const T &x)
    {
      constexpr double cf = dcoef(I);
      if constexpr (I == order - 1)
        return T(cf);
      else
        return hornerD<I + 1>(x) * x + T(cf);
    }
    template <int I, typename T> static GBINT_REG_HD T hornerdD(const T &x)  // D'(x), I from 1
    {
      constexpr double cf = I * dcoef(I);
      if constexpr (I >= order - 1)
        return T(cf);
      else
        return hornerdD<I + 1>(x) * x + T(cf);
    }

    template <typename T> static GBINT_REG_HD T get_f(const T x)
    {
      if constexpr (order == 1)
        return x;
      else
        return x * hornerP<1>(x) / hornerD<0>(x);
    }
    // f' = (P' D - P D') / D^2
    template <typename T> static GBINT_REG_HD T get_df(const T x)
    {
      if constexpr (order == 1)
        return T(1.);
      else {
        const T D = hornerD<0>(x);
        return (hornerdP<1>(x) * D - x * hornerP<1>(x) * hornerdD<1>(x)) / (D * D);
      }
    }

    template <typename NT1, typename NT2> static GBINT_REG_HD auto RB(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      const auto x = q2 / k2;
      return k2 * exp(-get_f(x));
    }
    // d/dt at fixed q^2: 2 k^2 e^(-f) (1 + x f'(x))
    template <typename NT1, typename NT2> static GBINT_REG_HD auto RBdot(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      const auto x = q2 / k2;
      return 2. * k2 * exp(-get_f(x)) * (1. + get_df(x) * x);
    }
    template <typename NT1, typename NT2> static GBINT_REG_HD auto dq2RB(const NT1 k2, const NT2 q2)
    {
      using std::exp;
      const auto x = q2 / k2;
      return -exp(-get_f(x)) * get_df(x);
    }
  };
} // namespace DiFfRG
