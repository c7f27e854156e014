// autodiff.hh -- first-order forward-mode numbers as integrator result types.
//
// DiFfRG instantiates its integrators with autodiff::real (the autodiff library's
// Real<1, double>: a value and one directional derivative), e.g.
//   Examples/ONfiniteT/flows/V/V.cu:17          IntegratorTBB<3, autodiff::real, V_kernel<...>>
//   DiFfRG/tests/physics/integration/integrator_1D_cartesian_gpu.cu:133-184
//                                               Integrator1DCartesianGPU<autodiff::real, ...>, checked
//                                               through autodiff::val / autodiff::derivative
// gbint::dual<T> plays that role for the class templates of gbint/integrators.hh: a KERNEL
// that takes dual arguments returns the integrand and its derivative along the seeded
// direction, and the integrator reduces both components (FP64 for T = double, compensated
// FP32 for T = float), so that get()/request() return the integral and its derivative.
// The arithmetic is the chain rule written out per operation; the derivative of every
// operation is exact up to the rounding of T.
//
// Code written against the autodiff library keeps working with it: specialise
// DiFfRG::gbint_detail::nt_traits and DiFfRG::get_type::ctype_of for its real type the same way
// as below (two components: value and derivative).
#pragma once

#include <cmath>
#include <type_traits>

#include <cuda/std/complex>

#include "gbint/integrators.hh"

namespace gbint
{
  template <typename T> struct dual;
  namespace ad_detail
  {
    template <typename T> struct is_cplx : std::false_type {
    };
    template <typename T> struct is_cplx<::cuda::std::complex<T>> : std::true_type {
    };
    // complex components: the elementary functions of cuda::std
    template <typename T> __host__ __device__ ::cuda::std::complex<T> exp_(const ::cuda::std::complex<T> &x)
    {
      return ::cuda::std::exp(x);
    }
    template <typename T> __host__ __device__ ::cuda::std::complex<T> log_(const ::cuda::std::complex<T> &x)
    {
      return ::cuda::std::log(x);
    }
    template <typename T> __host__ __device__ ::cuda::std::complex<T> sqrt_(const ::cuda::std::complex<T> &x)
    {
      return ::cuda::std::sqrt(x);
    }
    __host__ __device__ inline double exp_(double x) { return ::exp(x); }
    __host__ __device__ inline float exp_(float x) { return ::expf(x); }
    __host__ __device__ inline double expm1_(double x) { return ::expm1(x); }
    __host__ __device__ inline float expm1_(float x) { return ::expm1f(x); }
    __host__ __device__ inline double log_(double x) { return ::log(x); }
    __host__ __device__ inline float log_(float x) { return ::logf(x); }
    __host__ __device__ inline double log1p_(double x) { return ::log1p(x); }
    __host__ __device__ inline float log1p_(float x) { return ::log1pf(x); }
    __host__ __device__ inline double sqrt_(double x) { return ::sqrt(x); }
    __host__ __device__ inline float sqrt_(float x) { return ::sqrtf(x); }
    __host__ __device__ inline double sin_(double x) { return ::sin(x); }
    __host__ __device__ inline float sin_(float x) { return ::sinf(x); }
    __host__ __device__ inline double cos_(double x) { return ::cos(x); }
    __host__ __device__ inline float cos_(float x) { return ::cosf(x); }
    __host__ __device__ inline double tanh_(double x) { return ::tanh(x); }
    __host__ __device__ inline float tanh_(float x) { return ::tanhf(x); }
    __host__ __device__ inline double pow_(double x, double y) { return ::pow(x, y); }
    __host__ __device__ inline float pow_(float x, float y) { return ::powf(x, y); }
    __host__ __device__ inline double abs_(double x) { return ::fabs(x); }
    __host__ __device__ inline float abs_(float x) { return ::fabsf(x); }
    __host__ __device__ inline double sinh_(double x) { return ::sinh(x); }
    __host__ __device__ inline float sinh_(float x) { return ::sinhf(x); }
    __host__ __device__ inline double cosh_(double x) { return ::cosh(x); }
    __host__ __device__ inline float cosh_(float x) { return ::coshf(x); }
    __host__ __device__ inline double tan_(double x) { return ::tan(x); }
    __host__ __device__ inline float tan_(float x) { return ::tanf(x); }
    __host__ __device__ inline double atan_(double x) { return ::atan(x); }
    __host__ __device__ inline float atan_(float x) { return ::atanf(x); }
    __host__ __device__ inline double atan2_(double y, double x) { return ::atan2(y, x); }
    __host__ __device__ inline float atan2_(float y, float x) { return ::atan2f(y, x); }
    __host__ __device__ inline double asin_(double x) { return ::asin(x); }
    __host__ __device__ inline float asin_(float x) { return ::asinf(x); }
    __host__ __device__ inline double acos_(double x) { return ::acos(x); }
    __host__ __device__ inline float acos_(float x) { return ::acosf(x); }
  } // namespace ad_detail

  // value v and derivative d of a quantity along one seeded direction
  template <typename T> struct dual {
    static_assert(std::is_floating_point_v<T> || ad_detail::is_cplx<T>::value,
                  "gbint::dual<T> needs a floating-point or complex T");
    T v = 0, d = 0;

    constexpr dual() = default;
    __host__ __device__ constexpr dual(T value, T deriv) : v(value), d(deriv) {}
    // a constant (zero derivative): implicit, as for autodiff::real
    template <typename S, std::enable_if_t<std::is_arithmetic_v<S> || std::is_same_v<S, T>, int> = 0>
    __host__ __device__ constexpr dual(S value) : v(T(value)), d(0)
    {
    }
    template <typename U> __host__ __device__ constexpr explicit dual(const dual<U> &o) : v(T(o.v)), d(T(o.d)) {}
    // the value, by explicit conversion (as autodiff::real converts with a cast)
    __host__ __device__ constexpr explicit operator T() const { return v; }
    // component access in autodiff::real's layout: [0] the value, [1] the derivative
    __host__ __device__ T &operator[](int i) { return i ? d : v; }
    __host__ __device__ const T &operator[](int i) const { return i ? d : v; }

    __host__ __device__ dual &operator+=(const dual &b)
    {
      v += b.v;
      d += b.d;
      return *this;
    }
    __host__ __device__ dual &operator-=(const dual &b)
    {
      v -= b.v;
      d -= b.d;
      return *this;
    }
    __host__ __device__ dual &operator*=(const dual &b)
    {
      d = d * b.v + v * b.d;
      v *= b.v;
      return *this;
    }
    __host__ __device__ dual &operator/=(const dual &b)
    {
      const T r = T(1) / b.v;
      v *= r;
      d = (d - v * b.d) * r;
      return *this;
    }
  };

  // the value-and-derivative type of double results; under the reference's name it is
  // autodiff::real (bottom of this file)
  using dreal = dual<double>;

  template <typename T> __host__ __device__ constexpr T val(const dual<T> &a) { return a.v; }
  template <typename T> __host__ __device__ constexpr T derivative(const dual<T> &a) { return a.d; }
  // the seed of an independent variable: derivative 1
  template <typename T> __host__ __device__ constexpr dual<T> seed(T value) { return dual<T>(value, T(1)); }

  template <typename T> __host__ __device__ dual<T> operator+(const dual<T> &a) { return a; }
  template <typename T> __host__ __device__ dual<T> operator-(const dual<T> &a) { return dual<T>(-a.v, -a.d); }

  template <typename T> __host__ __device__ dual<T> operator+(dual<T> a, const dual<T> &b) { return a += b; }
  template <typename T> __host__ __device__ dual<T> operator-(dual<T> a, const dual<T> &b) { return a -= b; }
  template <typename T> __host__ __device__ dual<T> operator*(dual<T> a, const dual<T> &b) { return a *= b; }
  template <typename T> __host__ __device__ dual<T> operator/(dual<T> a, const dual<T> &b) { return a /= b; }

#define GBINT_DUAL_SCALAR_OPS(OP)                                                                          \
  template <typename T, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                   \
  __host__ __device__ dual<T> operator OP(const dual<T> &a, S s)                                         \
  {                                                                                                       \
    return a OP dual<T>(s);                                                                               \
  }                                                                                                       \
  template <typename T, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                   \
  __host__ __device__ dual<T> operator OP(S s, const dual<T> &a)                                         \
  {                                                                                                       \
    return dual<T>(s) OP a;                                                                               \
  }
  GBINT_DUAL_SCALAR_OPS(+)
  GBINT_DUAL_SCALAR_OPS(-)
  GBINT_DUAL_SCALAR_OPS(*)
  GBINT_DUAL_SCALAR_OPS(/)
#undef GBINT_DUAL_SCALAR_OPS

  // complex-valued forward numbers (the reference's cxReal, autodiff::Real<1, complex<double>>):
  // a real dual meeting a complex number or a complex dual becomes a complex dual
#define GBINT_DUAL_COMPLEX_OPS(OP)                                                                        \
  template <typename T>                                                                                   \
  __host__ __device__ dual<::cuda::std::complex<T>> operator OP(const dual<::cuda::std::complex<T>> &a,   \
                                                             const ::cuda::std::complex<T> &s)            \
  {                                                                                                       \
    return a OP dual<::cuda::std::complex<T>>(s);                                                        \
  }                                                                                                       \
  template <typename T>                                                                                   \
  __host__ __device__ dual<::cuda::std::complex<T>> operator OP(const ::cuda::std::complex<T> &s,         \
                                                             const dual<::cuda::std::complex<T>> &a)      \
  {                                                                                                       \
    return dual<::cuda::std::complex<T>>(s) OP a;                                                        \
  }                                                                                                       \
  template <typename T, std::enable_if_t<std::is_floating_point_v<T>, int> = 0>                           \
  __host__ __device__ dual<::cuda::std::complex<T>> operator OP(const dual<T> &a, const ::cuda::std::complex<T> &s) \
  {                                                                                                       \
    return dual<::cuda::std::complex<T>>(a) OP dual<::cuda::std::complex<T>>(s);                         \
  }                                                                                                       \
  template <typename T, std::enable_if_t<std::is_floating_point_v<T>, int> = 0>                           \
  __host__ __device__ dual<::cuda::std::complex<T>> operator OP(const ::cuda::std::complex<T> &s, const dual<T> &a) \
  {                                                                                                       \
    return dual<::cuda::std::complex<T>>(s) OP dual<::cuda::std::complex<T>>(a);                         \
  }                                                                                                       \
  template <typename T, std::enable_if_t<std::is_floating_point_v<T>, int> = 0>                           \
  __host__ __device__ dual<::cuda::std::complex<T>> operator OP(const dual<::cuda::std::complex<T>> &a,   \
                                                             const dual<T> &b)                            \
  {                                                                                                       \
    return a OP dual<::cuda::std::complex<T>>(b);                                                        \
  }                                                                                                       \
  template <typename T, std::enable_if_t<std::is_floating_point_v<T>, int> = 0>                           \
  __host__ __device__ dual<::cuda::std::complex<T>> operator OP(const dual<T> &a,                         \
                                                             const dual<::cuda::std::complex<T>> &b)      \
  {                                                                                                       \
    return dual<::cuda::std::complex<T>>(a) OP b;                                                        \
  }
  GBINT_DUAL_COMPLEX_OPS(+)
  GBINT_DUAL_COMPLEX_OPS(-)
  GBINT_DUAL_COMPLEX_OPS(*)
  GBINT_DUAL_COMPLEX_OPS(/)
#undef GBINT_DUAL_COMPLEX_OPS

  // real and imaginary parts: of a complex dual, component by component; of a real dual, itself and 0
  template <typename T> __host__ __device__ dual<T> real(const dual<::cuda::std::complex<T>> &a)
  {
    return dual<T>(a.v.real(), a.d.real());
  }
  template <typename T> __host__ __device__ dual<T> imag(const dual<::cuda::std::complex<T>> &a)
  {
    return dual<T>(a.v.imag(), a.d.imag());
  }
  template <typename T, std::enable_if_t<std::is_floating_point_v<T>, int> = 0>
  __host__ __device__ dual<T> real(const dual<T> &a)
  {
    return a;
  }
  template <typename T, std::enable_if_t<std::is_floating_point_v<T>, int> = 0>
  __host__ __device__ T imag(const dual<T> &)
  {
    return T(0);
  }

  template <typename T> __host__ __device__ bool operator<(const dual<T> &a, const dual<T> &b) { return a.v < b.v; }
  template <typename T> __host__ __device__ bool operator>(const dual<T> &a, const dual<T> &b) { return a.v > b.v; }
  template <typename T> __host__ __device__ bool operator==(const dual<T> &a, const dual<T> &b)
  {
    return a.v == b.v && a.d == b.d;
  }
  // comparisons with plain numbers compare the value
#define GBINT_DUAL_CMP(OP)                                                                                 \
  template <typename T, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                   \
  __host__ __device__ bool operator OP(const dual<T> &a, S s)                                            \
  {                                                                                                       \
    return a.v OP T(s);                                                                                   \
  }                                                                                                       \
  template <typename T, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>                   \
  __host__ __device__ bool operator OP(S s, const dual<T> &a)                                            \
  {                                                                                                       \
    return T(s) OP a.v;                                                                                   \
  }
  GBINT_DUAL_CMP(<)
  GBINT_DUAL_CMP(>)
  GBINT_DUAL_CMP(<=)
  GBINT_DUAL_CMP(>=)
#undef GBINT_DUAL_CMP
  template <typename T> __host__ __device__ bool operator<=(const dual<T> &a, const dual<T> &b) { return a.v <= b.v; }
  template <typename T> __host__ __device__ bool operator>=(const dual<T> &a, const dual<T> &b) { return a.v >= b.v; }

  // elementary functions: f(v), f'(v) d
  template <typename T> __host__ __device__ dual<T> exp(const dual<T> &a)
  {
    const T e = ad_detail::exp_(a.v);
    return dual<T>(e, e * a.d);
  }
  template <typename T> __host__ __device__ dual<T> expm1(const dual<T> &a)
  {
    return dual<T>(ad_detail::expm1_(a.v), ad_detail::exp_(a.v) * a.d);
  }
  template <typename T> __host__ __device__ dual<T> log(const dual<T> &a) { return dual<T>(ad_detail::log_(a.v), a.d / a.v); }
  template <typename T> __host__ __device__ dual<T> log1p(const dual<T> &a)
  {
    return dual<T>(ad_detail::log1p_(a.v), a.d / (T(1) + a.v));
  }
  template <typename T> __host__ __device__ dual<T> sqrt(const dual<T> &a)
  {
    const T s = ad_detail::sqrt_(a.v);
    return dual<T>(s, a.d / (T(2) * s));
  }
  template <typename T> __host__ __device__ dual<T> sin(const dual<T> &a)
  {
    return dual<T>(ad_detail::sin_(a.v), ad_detail::cos_(a.v) * a.d);
  }
  template <typename T> __host__ __device__ dual<T> cos(const dual<T> &a)
  {
    return dual<T>(ad_detail::cos_(a.v), -ad_detail::sin_(a.v) * a.d);
  }
  // tanh' = sech^2 = 1/cosh^2, accurate also where tanh rounds to +-1 (1 - tanh^2 would be 0 there)
  template <typename T> __host__ __device__ dual<T> tanh(const dual<T> &a)
  {
    const T c = ad_detail::cosh_(a.v);
    return dual<T>(ad_detail::tanh_(a.v), a.d / (c * c));
  }
  template <typename T> __host__ __device__ dual<T> abs(const dual<T> &a) { return a.v < 0 ? -a : a; }
  template <typename T> __host__ __device__ dual<T> fabs(const dual<T> &a) { return a.v < 0 ? -a : a; }
  template <typename T> __host__ __device__ dual<T> sinh(const dual<T> &a)
  {
    return dual<T>(ad_detail::sinh_(a.v), ad_detail::cosh_(a.v) * a.d);
  }
  template <typename T> __host__ __device__ dual<T> cosh(const dual<T> &a)
  {
    return dual<T>(ad_detail::cosh_(a.v), ad_detail::sinh_(a.v) * a.d);
  }
  // tan' = 1 + tan^2
  template <typename T> __host__ __device__ dual<T> tan(const dual<T> &a)
  {
    const T t = ad_detail::tan_(a.v);
    return dual<T>(t, (T(1) + t * t) * a.d);
  }
  template <typename T> __host__ __device__ dual<T> atan(const dual<T> &a)
  {
    return dual<T>(ad_detail::atan_(a.v), a.d / (T(1) + a.v * a.v));
  }
  // d atan2(y, x) = (x dy - y dx) / (x^2 + y^2)
  template <typename T> __host__ __device__ dual<T> atan2(const dual<T> &y, const dual<T> &x)
  {
    return dual<T>(ad_detail::atan2_(y.v, x.v), (x.v * y.d - y.v * x.d) / (x.v * x.v + y.v * y.v));
  }
  template <typename T, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
  __host__ __device__ dual<T> atan2(const dual<T> &y, S x)
  {
    return atan2(y, dual<T>(x));
  }
  template <typename T, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
  __host__ __device__ dual<T> atan2(S y, const dual<T> &x)
  {
    return atan2(dual<T>(y), x);
  }
  template <typename T> __host__ __device__ dual<T> asin(const dual<T> &a)
  {
    return dual<T>(ad_detail::asin_(a.v), a.d / ad_detail::sqrt_(T(1) - a.v * a.v));
  }
  template <typename T> __host__ __device__ dual<T> acos(const dual<T> &a)
  {
    return dual<T>(ad_detail::acos_(a.v), -a.d / ad_detail::sqrt_(T(1) - a.v * a.v));
  }
  template <typename T> __host__ __device__ bool isfinite(const dual<T> &a) { return ::isfinite(a.v) && ::isfinite(a.d); }
  template <typename T> __host__ __device__ bool isnan(const dual<T> &a) { return ::isnan(a.v) || ::isnan(a.d); }
  template <typename T, typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
  __host__ __device__ dual<T> pow(const dual<T> &a, S p)
  {
    const T e = T(p);
    const T r = ad_detail::pow_(a.v, e);
    return dual<T>(r, e * ad_detail::pow_(a.v, e - T(1)) * a.d);
  }
  template <typename T> __host__ __device__ dual<T> pow(const dual<T> &a, const dual<T> &b)
  {
    const T r = ad_detail::pow_(a.v, b.v);
    return dual<T>(r, r * (b.d * ad_detail::log_(a.v) + b.v * a.d / a.v));
  }
} // namespace gbint

namespace DiFfRG
{
  namespace get_type
  {
    template <typename T> struct ctype_of<gbint::dual<T>> {
      using type = T;
    };
  } // namespace get_type
  namespace gbint_detail
  {
    template <typename T> struct nt_traits<gbint::dual<T>> {
      static constexpr int C = 2;
      using S = T;
      __host__ __device__ static S get(const gbint::dual<T> &a, int c) { return c ? a.d : a.v; }
      static gbint::dual<T> make(const double *c) { return gbint::dual<T>(T(c[0]), T(c[1])); }
    };
  } // namespace gbint_detail
} // namespace DiFfRG

// autodiff::real, autodiff::Real<1, T>, autodiff::val and autodiff::derivative: the names
// DiFfRG code uses for the autodiff library's first-order forward numbers (e.g.
// Examples/ONfiniteT/flows/V/V.hh request<autodiff::real>), here gbint::dual.  A translation
// unit uses either this header or the autodiff library, not both.
namespace autodiff
{
  template <unsigned N, typename T> struct RealOrder;
  template <typename T> struct RealOrder<1, T> {
    using type = gbint::dual<T>;
  };
  template <unsigned N, typename T> using Real = typename RealOrder<N, T>::type;
  using real = gbint::dual<double>;
  using gbint::derivative;
  using gbint::val;
} // namespace autodiff
