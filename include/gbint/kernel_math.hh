// kernel_math.hh -- the arithmetic helpers generated DiFfRG KERNELs call, without the
// reference's Eigen/autodiff/deal.II includes: powr<n> (DiFfRG/include/DiFfRG/common/math.hh:40-54,
// x^n by the same right-nested products, 1/x^-n for n < 0) and the complex type of
// DiFfRG/include/DiFfRG/common/complex_math.hh (cuda::std::complex on host and device).
// A KERNEL file that includes DiFfRG/common/math.hh and complex_math.hh from a DiFfRG
// installation does not need this header; one that is built without them includes it instead.
#pragma once

#include <type_traits>

#include <cuda/std/complex>

namespace DiFfRG
{
  template <int n, typename NumberType> constexpr __forceinline__ __host__ __device__ NumberType powr(const NumberType x)
  {
    if constexpr (n == 0)
      return NumberType(1.);
    else if constexpr (n < 0)
      return NumberType(1.) / powr<-n, NumberType>(x);
    else if constexpr (n > 1)
      return x * powr<n - 1, NumberType>(x);
    else
      return x;
  }

  // the complex type and its accessors; the elementary functions of a complex argument are found
  // by argument-dependent lookup in cuda::std, those of a real one are the usual ones (bringing
  // cuda::std's real overloads into this namespace would make ::sqrt(double) ambiguous in code
  // that uses namespace DiFfRG)
  using ::cuda::std::complex;
  using ::cuda::std::imag;
  using ::cuda::std::real;
  template <typename NT> constexpr __host__ __device__ auto cot(const NT x) { return NT(1) / tan(x); }
} // namespace DiFfRG
