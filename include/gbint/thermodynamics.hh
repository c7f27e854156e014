// thermodynamics.hh -- the hyperbolic and distribution-function helpers generated finite-T
// KERNELs call, host and device, for real, complex and gbint::dual arguments.
//
// Names and meanings follow DiFfRG/include/DiFfRG/physics/thermodynamics.hh:12-135 (generated
// kernels call them by these names, e.g. Examples/ONfiniteT/flows/V/V.kernel):
//   Cosh Sinh Tanh Coth Sech Csch                 the hyperbolic functions by capitalised name
//   CothFiniteT(x, T) = coth(x / 2T)              sign(Re x) in the limit T/x -> 0 (T = 0 included)
//   TanhFiniteT(x, T) = tanh(x / 2T)              same limit
//   SechFiniteT(x, T) = 1/cosh(x / 2T)            0 where cosh(x/2T) overflows
//   CschFiniteT(x, T) = 1/sinh(x / 2T)            same
//   cothS tanhS sechS cschS (e, T)                coth, tanh, sech, csch of e/(2T)
//   dcothS ddcothS dddcothS dtanhS ddtanhS        their derivatives in e, from d/du coth u = -csch^2 u,
//                                                 d/du tanh u = sech^2 u and the chain rule (u = e/2T)
//   nB(e, T) = 1/(e^{e/T} - 1), nF(e, T) = 1/(e^{e/T} + 1), dnB, ddnB, dnF   and their e-derivatives
// The limit test of the FiniteT forms treats T/x as zero when |T| <= eps |x| with eps the double
// epsilon (the reference asks whether T/x is close to 0 at that epsilon).
#pragma once

#include <cmath>
#include <limits>
#include <type_traits>

#include <cuda/std/complex>

#ifndef GBINT_TD_HD
#define GBINT_TD_HD __host__ __device__ __forceinline__
#endif

namespace DiFfRG
{
  namespace gbint_td
  {
    template <typename T> GBINT_TD_HD double re(const T &x) { return (double)x; }
    template <typename T> GBINT_TD_HD double re(const ::cuda::std::complex<T> &x) { return (double)x.real(); }
    template <typename T> GBINT_TD_HD double mag(const T &x) { return ::fabs(re(x)); }
    template <typename T> GBINT_TD_HD double mag(const ::cuda::std::complex<T> &x)
    {
      return (double)::cuda::std::abs(x);
    }
    template <typename T> GBINT_TD_HD bool finite(const T &x) { return ::isfinite(re(x)); }
    template <typename T> GBINT_TD_HD bool finite(const ::cuda::std::complex<T> &x)
    {
      return ::isfinite((double)x.real()) && ::isfinite((double)x.imag());
    }
    // T/x treated as 0
    template <typename X, typename TT> GBINT_TD_HD bool zero_T_over_x(const X &x, TT T)
    {
      return ::fabs((double)T) <= std::numeric_limits<double>::epsilon() * mag(x);
    }
  } // namespace gbint_td

  using std::cosh, std::sinh, std::tanh, std::exp, std::expm1;

  template <typename T> GBINT_TD_HD auto Cosh(const T x) { return cosh(x); }
  template <typename T> GBINT_TD_HD auto Sinh(const T x) { return sinh(x); }
  template <typename T> GBINT_TD_HD auto Tanh(const T x) { return tanh(x); }
  template <typename T> GBINT_TD_HD auto Coth(const T x) { return 1. / tanh(x); }
  template <typename T> GBINT_TD_HD auto Sech(const T x) { return 1. / cosh(x); }
  template <typename T> GBINT_TD_HD auto Csch(const T x) { return 1. / sinh(x); }

  template <typename T1, typename T2, std::enable_if_t<std::is_arithmetic_v<T2>, int> = 0>
  GBINT_TD_HD auto CothFiniteT(const T1 x, const T2 T)
  {
    using R = decltype(Coth(x / (2 * T)));
    if (gbint_td::zero_T_over_x(x, T)) return (R)(gbint_td::re(x) < 0 ? -1 : 1);
    return (R)Coth(x / (2 * T));
  }
  template <typename T1, typename T2, std::enable_if_t<std::is_arithmetic_v<T2>, int> = 0>
  GBINT_TD_HD auto TanhFiniteT(const T1 x, const T2 T)
  {
    using R = decltype(Tanh(x / (2 * T)));
    if (gbint_td::zero_T_over_x(x, T)) return (R)(gbint_td::re(x) < 0 ? -1 : 1);
    return (R)Tanh(x / (2 * T));
  }
  template <typename T1, typename T2, std::enable_if_t<std::is_arithmetic_v<T2>, int> = 0>
  GBINT_TD_HD auto SechFiniteT(const T1 x, const T2 T)
  {
    const auto c = Cosh(x / (2 * T));
    using R = decltype(c);
    return gbint_td::finite(c) ? (R)(R(1) / c) : (R)0;
  }
  template <typename T1, typename T2, std::enable_if_t<std::is_arithmetic_v<T2>, int> = 0>
  GBINT_TD_HD auto CschFiniteT(const T1 x, const T2 T)
  {
    const auto s = Sinh(x / (2 * T));
    using R = decltype(s);
    return gbint_td::finite(s) ? (R)(R(1) / s) : (R)0;
  }

  // functions of u = e / (2T) and their e-derivatives (du/de = 1/(2T))
  template <typename T1, typename T2> GBINT_TD_HD auto cothS(const T1 e, const T2 T) { return 1. / tanh(e / (T * 2.)); }
  template <typename T1, typename T2> GBINT_TD_HD auto tanhS(const T1 e, const T2 T) { return tanh(e / (T * 2.)); }
  template <typename T1, typename T2> GBINT_TD_HD auto sechS(const T1 e, const T2 T) { return 1. / cosh(e / (T * 2.)); }
  template <typename T1, typename T2> GBINT_TD_HD auto cschS(const T1 e, const T2 T) { return 1. / sinh(e / (T * 2.)); }
  // d/de coth(u) = -csch^2(u) / (2T)
  template <typename T1, typename T2> GBINT_TD_HD auto dcothS(const T1 e, const T2 T)
  {
    const auto c = cschS(e, T);
    return -(c * c) / (2. * T);
  }
  // d^2/de^2 coth(u): d/de(-csch^2 u / 2T) = csch^2(u) coth(u) / (2 T^2) = -dcothS coth / T
  template <typename T1, typename T2> GBINT_TD_HD auto ddcothS(const T1 e, const T2 T)
  {
    return -dcothS(e, T) * cothS(e, T) / T;
  }
  // d^3/de^3 coth(u) = -(ddcothS coth + dcothS d(coth)/de) / T with d(coth)/de = dcothS;
  // written with the product rule in e
  template <typename T1, typename T2> GBINT_TD_HD auto dddcothS(const T1 e, const T2 T)
  {
    const auto d1 = dcothS(e, T);
    return -(ddcothS(e, T) * cothS(e, T) + d1 * d1) / T;
  }
  // d/de tanh(u) = sech^2(u) / (2T)
  template <typename T1, typename T2> GBINT_TD_HD auto dtanhS(const T1 e, const T2 T)
  {
    const auto s = sechS(e, T);
    return (s * s) / (2. * T);
  }
  // d^2/de^2 tanh(u) = -2 sech^2(u) tanh(u) / (4 T^2) = -dtanhS tanh / T
  template <typename T1, typename T2> GBINT_TD_HD auto ddtanhS(const T1 e, const T2 T)
  {
    return -dtanhS(e, T) * tanhS(e, T) / T;
  }

  // Bose-Einstein and Fermi-Dirac distributions and their e-derivatives
  template <typename T1, typename T2> GBINT_TD_HD auto nB(const T1 e, const T2 T) { return 1. / expm1(e / T); }
  // d/de (e^{e/T} - 1)^{-1} = -e^{e/T} / (T (e^{e/T} - 1)^2)
  template <typename T1, typename T2> GBINT_TD_HD auto dnB(const T1 e, const T2 T)
  {
    const auto m = expm1(e / T);
    return -exp(e / T) / (m * m) / T;
  }
  // d^2/de^2: e^{e/T} (e^{e/T} + 1) / (T^2 (e^{e/T} - 1)^3)
  template <typename T1, typename T2> GBINT_TD_HD auto ddnB(const T1 e, const T2 T)
  {
    const auto x = exp(e / T);
    const auto m = expm1(e / T);
    return x * (1. + x) / (m * m * m) / (T * T);
  }
  template <typename T1, typename T2> GBINT_TD_HD auto nF(const T1 e, const T2 T) { return 1. / (exp(e / T) + 1.); }
  // d/de (e^{e/T} + 1)^{-1} = -e^{e/T} / (T (e^{e/T} + 1)^2)
  template <typename T1, typename T2> GBINT_TD_HD auto dnF(const T1 e, const T2 T)
  {
    const auto x = exp(e / T);
    const auto p = x + 1.;
    return -x / (p * p) / T;
  }
} // namespace DiFfRG
