// math_compat.hh -- the numeric helpers of DiFfRG/include/DiFfRG/common/math.hh and
// complex_math.hh that generated flows and their host code use, without Eigen, deal.II or the
// autodiff library:
//   powr<n>, complex, real, imag, cot        (gbint/kernel_math.hh)
//   V_d(d[, extent]), S_d(d), S_d_prec<NT>(d) volume and surface of the unit d-ball/-sphere
//   heaviside_theta(x), sign(x)              1 for x >= 0 (else 0 resp. -1), as the reference defines them
//   is_close(a, b[, eps])                    |a-b| <= eps or |a-b| <= eps max(|a|,|b|); complex parts
//                                            separately; eps defaults to the larger type epsilon
//                                            (10 double epsilons when a dual number is involved)
//   dot<n, NT>(a1, a2)                       sum of n products
//   is_complex<T>                            trait
//   mixed-type complex arithmetic            float (x) complex<double> etc., as complex_math.hh:78-124
//   autodiff::real, val, derivative           forward-mode numbers (gbint::dual, gbint/autodiff.hh)
//                                            under the names generated code uses: autodiff::real is
//                                            the result type of e.g. Examples/ONfiniteT/flows/V/V.hh
#pragma once

#include <cmath>
#include <limits>
#include <type_traits>

#include <cuda/std/complex>

#include "gbint/autodiff.hh"
#include "gbint/kernel_math.hh"

namespace DiFfRG
{
  using std::isfinite;
  using gbint::isfinite;

  template <typename T> struct is_complex : std::false_type {
  };
  template <typename T> struct is_complex<::cuda::std::complex<T>> : std::true_type {
  };
  template <typename T> struct is_dual : std::false_type {
  };
  template <typename T> struct is_dual<gbint::dual<T>> : std::true_type {
  };

  template <typename NT> __host__ __device__ inline double V_d(NT d)
  {
    return ::pow(M_PI, d / 2.) / ::tgamma(d / 2. + 1.);
  }
  template <typename NT1, typename NT2> __host__ __device__ inline double V_d(NT1 d, NT2 extent)
  {
    return ::pow(M_PI, d / 2.) / ::tgamma(d / 2. + 1.) * ::pow(extent, d);
  }
  template <typename NT> __host__ __device__ inline double S_d(NT d) { return 2. * ::pow(M_PI, d / 2.) / ::tgamma(d / 2.); }
  // S_d in the precision of NT, from its closed forms for d <= 7 (NaN beyond)
  template <typename NT> constexpr NT S_d_prec(unsigned d)
  {
    const NT pi = static_cast<NT>(M_PI);
    switch (d) {
    case 1: return NT(2);
    case 2: return NT(2) * pi;
    case 3: return NT(4) * pi;
    case 4: return NT(2) * pi * pi;
    case 5: return NT(8) * pi * pi / NT(3);
    case 6: return pi * pi * pi;
    case 7: return NT(16) * pi * pi * pi / NT(15);
    }
    return std::numeric_limits<NT>::quiet_NaN();
  }

  template <typename NumberType> __host__ __device__ constexpr auto heaviside_theta(const NumberType x)
  {
    if constexpr (is_dual<NumberType>::value)
      return x >= 0. ? 1. : 0.;
    else
      return x >= static_cast<NumberType>(0) ? static_cast<NumberType>(1) : static_cast<NumberType>(0);
  }
  template <typename NumberType> __host__ __device__ constexpr auto sign(const NumberType x)
  {
    if constexpr (is_dual<NumberType>::value)
      return x >= 0. ? 1. : -1.;
    else
      return x >= static_cast<NumberType>(0) ? static_cast<NumberType>(1) : static_cast<NumberType>(-1);
  }

  namespace gbint_math
  {
    template <typename T> constexpr double eps_of()
    {
      if constexpr (is_complex<T>::value)
        return std::numeric_limits<typename T::value_type>::epsilon();
      else if constexpr (is_dual<T>::value)
        return 10. * std::numeric_limits<double>::epsilon();
      else
        return std::numeric_limits<T>::epsilon();
    }
    template <typename T> constexpr bool closeable()
    {
      return std::is_floating_point_v<T> || is_complex<T>::value || is_dual<T>::value;
    }
  } // namespace gbint_math

  template <typename T1, typename T2, typename T3,
            std::enable_if_t<gbint_math::closeable<T1>() && gbint_math::closeable<T2>() &&
                                 std::is_floating_point_v<T3>,
                             int> = 0>
  __host__ __device__ bool is_close(T1 a, T2 b, T3 eps_)
  {
    if constexpr (is_complex<T1>::value || is_complex<T2>::value) {
      return is_close((double)::cuda::std::real(a), (double)::cuda::std::real(b), (double)eps_) &&
             is_close((double)::cuda::std::imag(a), (double)::cuda::std::imag(b), (double)eps_);
    } else if constexpr (is_dual<T1>::value || is_dual<T2>::value) {
      return is_close((double)a, (double)b, (double)eps_);
    } else {
      const auto diff = ::fabs(a - b);
      if (diff <= eps_) return true;
      return diff <= ::fmax(::fabs(a), ::fabs(b)) * eps_;
    }
  }
  template <typename T1, typename T2,
            std::enable_if_t<gbint_math::closeable<T1>() && gbint_math::closeable<T2>(), int> = 0>
  __host__ __device__ bool is_close(T1 a, T2 b)
  {
    constexpr double e1 = gbint_math::eps_of<T1>(), e2 = gbint_math::eps_of<T2>();
    if constexpr (is_dual<T1>::value || is_dual<T2>::value)
      return is_close(a, b, 10. * std::numeric_limits<double>::epsilon());
    else
      return is_close(a, b, e1 > e2 ? e1 : e2);
  }

  template <unsigned n, typename NT, typename A1, typename A2> NT dot(const A1 &a1, const A2 &a2)
  {
    NT ret = a1[0] * a2[0];
    for (unsigned i = 1; i < n; ++i) ret += a1[i] * a2[i];
    return ret;
  }

  // complex arithmetic with a real of another type (cuda::std::complex takes only its own type)
  template <typename T1, typename T2,
            std::enable_if_t<!std::is_same_v<T1, T2> && std::is_arithmetic_v<T1> && std::is_arithmetic_v<T2>, int> = 0>
  __host__ __device__ auto operator*(const T1 x, const ::cuda::std::complex<T2> &y)
  {
    using R = decltype(T1(1) * T2(1));
    return ::cuda::std::complex<R>(R(x) * R(y.real()), R(x) * R(y.imag()));
  }
  template <typename T1, typename T2,
            std::enable_if_t<!std::is_same_v<T1, T2> && std::is_arithmetic_v<T1> && std::is_arithmetic_v<T2>, int> = 0>
  __host__ __device__ auto operator*(const ::cuda::std::complex<T1> &x, const T2 y)
  {
    using R = decltype(T1(1) * T2(1));
    return ::cuda::std::complex<R>(R(x.real()) * R(y), R(x.imag()) * R(y));
  }
  template <typename T1, typename T2,
            std::enable_if_t<!std::is_same_v<T1, T2> && std::is_arithmetic_v<T1> && std::is_arithmetic_v<T2>, int> = 0>
  __host__ __device__ auto operator+(const T1 x, const ::cuda::std::complex<T2> &y)
  {
    using R = decltype(T1(1) + T2(1));
    return ::cuda::std::complex<R>(R(x) + R(y.real()), R(y.imag()));
  }
  template <typename T1, typename T2,
            std::enable_if_t<!std::is_same_v<T1, T2> && std::is_arithmetic_v<T1> && std::is_arithmetic_v<T2>, int> = 0>
  __host__ __device__ auto operator+(const ::cuda::std::complex<T1> &x, const T2 y)
  {
    using R = decltype(T1(1) + T2(1));
    return ::cuda::std::complex<R>(R(x.real()) + R(y), R(x.imag()));
  }
  template <typename T1, typename T2,
            std::enable_if_t<!std::is_same_v<T1, T2> && std::is_arithmetic_v<T1> && std::is_arithmetic_v<T2>, int> = 0>
  __host__ __device__ auto operator-(const T1 x, const ::cuda::std::complex<T2> &y)
  {
    using R = decltype(T1(1) - T2(1));
    return ::cuda::std::complex<R>(R(x) - R(y.real()), -R(y.imag()));
  }
  template <typename T1, typename T2,
            std::enable_if_t<!std::is_same_v<T1, T2> && std::is_arithmetic_v<T1> && std::is_arithmetic_v<T2>, int> = 0>
  __host__ __device__ auto operator-(const ::cuda::std::complex<T1> &x, const T2 y)
  {
    using R = decltype(T1(1) - T2(1));
    return ::cuda::std::complex<R>(R(x.real()) - R(y), R(x.imag()));
  }
  // x / y = x conj(y) / |y|^2
  template <typename T1, typename T2,
            std::enable_if_t<!std::is_same_v<T1, T2> && std::is_arithmetic_v<T1> && std::is_arithmetic_v<T2>, int> = 0>
  __host__ __device__ auto operator/(const T1 x, const ::cuda::std::complex<T2> &y)
  {
    using R = decltype(T1(1) / T2(1));
    const R n = R(y.real()) * R(y.real()) + R(y.imag()) * R(y.imag());
    return ::cuda::std::complex<R>(R(x) * R(y.real()) / n, -R(x) * R(y.imag()) / n);
  }
  template <typename T1, typename T2,
            std::enable_if_t<!std::is_same_v<T1, T2> && std::is_arithmetic_v<T1> && std::is_arithmetic_v<T2>, int> = 0>
  __host__ __device__ auto operator/(const ::cuda::std::complex<T1> &x, const T2 y)
  {
    using R = decltype(T1(1) / T2(1));
    return ::cuda::std::complex<R>(R(x.real()) / R(y), R(x.imag()) / R(y));
  }
} // namespace DiFfRG
