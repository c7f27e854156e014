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

#include "gbint/integrators.hh"

namespace gbint
{
  namespace ad_detail
  {
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
  } // namespace ad_detail

  // value v and derivative d of a quantity along one seeded direction
  template <typename T> struct dual {
    static_assert(std::is_floating_point_v<T>, "gbint::dual<T> needs a floating-point T");
    T v = 0, d = 0;

    __host__ __device__ constexpr dual() = default;
    __host__ __device__ constexpr dual(T value, T deriv) : v(value), d(deriv) {}
    // a constant (zero derivative): implicit, as for autodiff::real
    template <typename S, std::enable_if_t<std::is_arithmetic_v<S>, int> = 0>
    __host__ __device__ constexpr dual(S value) : v(T(value)), d(0)
    {
    }
    template <typename U> __host__ __device__ constexpr explicit dual(const dual<U> &o) : v(T(o.v)), d(T(o.d)) {}

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

  using real = dual<double>;

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
  template <typename T> __host__ __device__ dual<T> tanh(const dual<T> &a)
  {
    const T t = ad_detail::tanh_(a.v);
    return dual<T>(t, (T(1) - t * t) * a.d);
  }
  template <typename T> __host__ __device__ dual<T> abs(const dual<T> &a) { return a.v < 0 ? -a : a; }
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
