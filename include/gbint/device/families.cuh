// families.cuh -- device code of the C++ class templates: one integrand point of every
// integrator family, with the reference's maps and Jacobians, for a user KERNEL.
//
// Each family F provides
//   points(P)                       number of grid points of the flattened tensor grid
//   eval<KERNEL, NT>(P, idx, t...)  weight * KERNEL::kernel(coordinates..., k, t...) at point idx
//                                   (both signs of q0 where the reference evaluates both)
// over the provider's Gauss-Legendre arrays on [0,1] (and Matsubara arrays), so the k-dependent
// maps are applied per point as the reference kernels do, e.g. q = k sqrt(x x_extent),
// cos = 2(t - 1/2), phi = 2 pi t (integrator_4D_gpu.hh:32-47).  Sources per family below.
// Every angular axis has its own rule and order (the reference requires equal angular orders).
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace gbint
{
  namespace fam
  {
    template <typename ctype> struct Params {
      const ctype *x[4] = {nullptr, nullptr, nullptr, nullptr};  // GL nodes on [0,1] per axis
      const ctype *w[4] = {nullptr, nullptr, nullptr, nullptr};
      int n[4] = {0, 0, 0, 0};
      const ctype *mx = nullptr, *mw = nullptr;  // Matsubara nodes / weights
      int nm = 0;
      ctype k = 1, x_extent = 1, x0_extent = 0, T = 0;
      int ns = 0;  // explicit Matsubara summands (x0 families; 0 at T = 0)
      ctype log_start = 0, log_ext = 0, off = 0;
      ctype qmin[3] = {0, 0, 0}, qext[3] = {0, 0, 0};
    };

    template <typename ctype> __host__ __device__ __forceinline__ ctype powi(ctype x, int n)
    {
      ctype r = 1;
      if (n < 0) {
        for (int i = 0; i < -n; ++i) r /= x;
        return r;
      }
      for (int i = 0; i < n; ++i) r *= x;
      return r;
    }
    // S_d of DiFfRG/include/DiFfRG/common/math.hh:104-121
    template <typename ctype> __host__ __device__ __forceinline__ ctype S_d(int d)
    {
      const ctype pi = (ctype)3.14159265358979323846;
      switch (d) {
      case 1: return 2;
      case 2: return 2 * pi;
      case 3: return 4 * pi;
      case 4: return 2 * pi * pi;
      case 5: return 8 * pi * pi / 3;
      case 6: return pi * pi * pi;
      case 7: return 16 * pi * pi * pi / 15;
      }
      return (ctype)NAN;
    }
    template <typename ctype> __host__ __device__ __forceinline__ ctype two_pi() { return (ctype)6.283185307179586476925; }

    // IntegratorGPU<d>: gridreduce functor, integrator_gpu.hh:34-60
    template <int d> struct F1D {
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P) { return P.n[0]; }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const int i = (int)idx;
        const ctype q = P.k * sqrt(P.x[0][i] * P.x_extent);
        const ctype ie = S_d<ctype>(d) * (powi(q, d - 2) / (ctype)2 * P.k * P.k) / powi(two_pi<ctype>(), d);
        return ie * P.w[0][i] * P.x_extent * K::kernel(q, P.k, t...);
      }
    };

    // IntegratorAngleGPU<d>: gridreduce_angle, integrator_angle_gpu.hh:21-40
    template <int d> struct FAngle {
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P)
      {
        return (long long)P.n[0] * P.n[1];
      }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const int i = (int)(idx / P.n[1]), j = (int)(idx % P.n[1]);
        const ctype q = P.k * sqrt(P.x[0][i] * P.x_extent);
        const ctype cs = 2 * (P.x[1][j] - (ctype)0.5);
        const ctype ie = S_d<ctype>(d) * (powi(q, d - 2) / (ctype)2 * P.k * P.k) * ((ctype)1 / 2) /
                         powi(two_pi<ctype>(), d);
        const ctype wt = 2 * P.w[1][j] * P.w[0][i] * P.x_extent;
        return ie * wt * K::kernel(q, cs, P.k, t...);
      }
    };

    // Integrator3DGPU: gridreduce_3d, integrator_3D_gpu.hh:21-43
    struct F3D {
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P)
      {
        return (long long)P.n[0] * P.n[1] * P.n[2];
      }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const int l = (int)(idx % P.n[2]);
        idx /= P.n[2];
        const int j = (int)(idx % P.n[1]), i = (int)(idx / P.n[1]);
        const ctype q = P.k * sqrt(P.x[0][i] * P.x_extent);
        const ctype cs = 2 * (P.x[1][j] - (ctype)0.5);
        const ctype phi = two_pi<ctype>() * P.x[2][l];
        const ctype ie = (q / (ctype)2 * P.k * P.k) / powi(two_pi<ctype>(), 3);
        const ctype wt = two_pi<ctype>() * P.w[2][l] * 2 * P.w[1][j] * P.w[0][i] * P.x_extent;
        return ie * wt * K::kernel(q, cs, phi, P.k, t...);
      }
    };

    // Integrator4D2AngGPU: gridreduce_4d_2ang, integrator_4D_2ang_gpu.hh:21-45
    struct F4D2Ang {
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P)
      {
        return (long long)P.n[0] * P.n[1] * P.n[2];
      }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const int l = (int)(idx % P.n[2]);
        idx /= P.n[2];
        const int j = (int)(idx % P.n[1]), i = (int)(idx / P.n[1]);
        const ctype q = P.k * sqrt(P.x[0][i] * P.x_extent);
        const ctype c1 = 2 * (P.x[1][j] - (ctype)0.5), c2 = 2 * (P.x[2][l] - (ctype)0.5);
        const ctype ie = two_pi<ctype>() * (q * q * (ctype)0.5 * P.k * P.k) * sqrt(1 - c1 * c1) /
                         powi(two_pi<ctype>(), 4);
        const ctype wt = 2 * P.w[2][l] * 2 * P.w[1][j] * P.w[0][i] * P.x_extent;
        return ie * wt * K::kernel(q, c1, c2, P.k, t...);
      }
    };

    // Integrator4DGPU: gridreduce_4d, integrator_4D_gpu.hh:21-49 (cos2 with its own order)
    struct F4D {
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P)
      {
        return (long long)P.n[0] * P.n[1] * P.n[2] * P.n[3];
      }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const int m = (int)(idx % P.n[3]);
        idx /= P.n[3];
        const int l = (int)(idx % P.n[2]);
        idx /= P.n[2];
        const int j = (int)(idx % P.n[1]), i = (int)(idx / P.n[1]);
        const ctype q = P.k * sqrt(P.x[0][i] * P.x_extent);
        const ctype c1 = 2 * (P.x[1][j] - (ctype)0.5), c2 = 2 * (P.x[2][l] - (ctype)0.5);
        const ctype phi = two_pi<ctype>() * P.x[3][m];
        const ctype ie = (q * q * (ctype)0.5 * P.k * P.k) * sqrt(1 - c1 * c1) / powi(two_pi<ctype>(), 4);
        const ctype wt = two_pi<ctype>() * P.w[3][m] * 2 * P.w[2][l] * 2 * P.w[1][j] * P.w[0][i] * P.x_extent;
        return ie * wt * K::kernel(q, c1, c2, phi, P.k, t...);
      }
    };

    // Integrator{1,2,3}DCartesianGPU: integrator_*D_cartesian_gpu.hh (e.g. 2D at :28-46)
    template <int dim> struct FCart {
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P)
      {
        long long p = P.n[0];
        if (dim > 1) p *= P.n[1];
        if (dim > 2) p *= P.n[2];
        return p;
      }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const ctype ie = powi(two_pi<ctype>(), -dim);
        if constexpr (dim == 1) {
          const int i = (int)idx;
          const ctype qx = P.qmin[0] + P.qext[0] * P.x[0][i];
          return ie * P.qext[0] * P.w[0][i] * K::kernel(qx, P.k, t...);
        } else if constexpr (dim == 2) {
          const int j = (int)(idx % P.n[1]), i = (int)(idx / P.n[1]);
          const ctype qx = P.qmin[0] + P.qext[0] * P.x[0][i], qy = P.qmin[1] + P.qext[1] * P.x[1][j];
          return ie * P.qext[1] * P.w[1][j] * P.qext[0] * P.w[0][i] * K::kernel(qx, qy, P.k, t...);
        } else {
          const int l = (int)(idx % P.n[2]);
          idx /= P.n[2];
          const int j = (int)(idx % P.n[1]), i = (int)(idx / P.n[1]);
          const ctype qx = P.qmin[0] + P.qext[0] * P.x[0][i], qy = P.qmin[1] + P.qext[1] * P.x[1][j];
          const ctype qz = P.qmin[2] + P.qext[2] * P.x[2][l];
          return ie * P.qext[2] * P.w[2][l] * P.qext[1] * P.w[1][j] * P.qext[0] * P.w[0][i] *
                 K::kernel(qx, qy, qz, P.k, t...);
        }
      }
    };

    // Integrator2Dp{q,x}0GPU: gridreduce_2dp{q,x}0, integrator_2Dpq0_gpu.hh:21-46, integrator_2Dpx0_gpu.hh:28-54
    template <bool PX> struct F2Dp0 {
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P)
      {
        return (long long)P.n[0] * P.n[1] * P.n[2];
      }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const int l = (int)(idx % P.n[2]);
        idx /= P.n[2];
        const int j = (int)(idx % P.n[1]), i = (int)(idx / P.n[1]);
        const ctype q = P.k * sqrt(P.x[0][i] * P.x_extent);
        const ctype cs = 2 * (P.x[1][j] - (ctype)0.5);
        const ctype q0 = (PX ? P.k : (ctype)1) * P.x[2][l] * P.x0_extent;
        const ctype ie = ((ctype)1 / 2 * P.k * P.k) * two_pi<ctype>() * ((ctype)1 / 2) * (PX ? P.k : (ctype)1) /
                         powi(two_pi<ctype>(), 3);
        const ctype wt = P.w[2][l] * P.x0_extent * 2 * P.w[1][j] * P.w[0][i] * P.x_extent;
        return ie * wt * (K::kernel(q, cs, q0, P.k, t...) + K::kernel(q, cs, -q0, P.k, t...));
      }
    };

    // Integrator3Dp{q,x}0GPU: gridreduce_3dp{q,x}0, integrator_3Dpq0_gpu.hh:21-46 (phi, q0 own orders)
    template <bool PX> struct F3Dp0 {
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P)
      {
        return (long long)P.n[0] * P.n[1] * P.n[2] * P.n[3];
      }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const int m = (int)(idx % P.n[3]);
        idx /= P.n[3];
        const int l = (int)(idx % P.n[2]);
        idx /= P.n[2];
        const int j = (int)(idx % P.n[1]), i = (int)(idx / P.n[1]);
        const ctype q = P.k * sqrt(P.x[0][i] * P.x_extent);
        const ctype cs = 2 * (P.x[1][j] - (ctype)0.5);
        const ctype phi = two_pi<ctype>() * P.x[2][l];
        const ctype q0 = (PX ? P.k : (ctype)1) * P.x[3][m] * P.x0_extent;
        const ctype ie = (q / (ctype)2 * P.k * P.k) * (PX ? P.k : (ctype)1) / powi(two_pi<ctype>(), 4);
        const ctype wt = P.w[3][m] * P.x0_extent * two_pi<ctype>() * P.w[2][l] * 2 * P.w[1][j] * P.w[0][i] * P.x_extent;
        return ie * wt * (K::kernel(q, cs, phi, q0, P.k, t...) + K::kernel(q, cs, phi, -q0, P.k, t...));
      }
    };

    // Integrator{,Angle,4D}FiniteTq0GPU: T f(0) + sum_i w_i [f(x_i) + f(-x_i)]
    // (integrator_finiteTq0_gpu.hh:21-44, integrator_angle_finiteTq0_gpu.hh:21-50, integrator_4D_finiteTq0_gpu.hh:21-55)
    template <int d, int ANG> struct FTq0 {  // ANG: 0 radial only, 1 cos, 2 cos + phi (d = 4)
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P)
      {
        long long p = (long long)P.n[0] * P.nm;
        if (ANG >= 1) p *= P.n[1];
        if (ANG == 2) p *= P.n[2];
        return p;
      }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const int m = (int)(idx % P.nm);
        idx /= P.nm;
        int l = 0, j = 0;
        if (ANG == 2) {
          l = (int)(idx % P.n[2]);
          idx /= P.n[2];
        }
        if (ANG >= 1) {
          j = (int)(idx % P.n[1]);
          idx /= P.n[1];
        }
        const int i = (int)idx;
        const ctype q = P.k * sqrt(P.x[0][i] * P.x_extent);
        ctype ie;
        if (ANG == 2)
          ie = (q / (ctype)2 * P.k * P.k) / powi(two_pi<ctype>(), 3);
        else
          ie = S_d<ctype>(d - 1) * (powi(q, d - 3) / (ctype)2 * P.k * P.k) * (ANG == 1 ? (ctype)0.5 : (ctype)1) /
               powi(two_pi<ctype>(), d - 1);
        ctype xw = P.w[0][i] * P.x_extent;
        const ctype q0 = P.mx[m];
        NT v;
        if constexpr (ANG == 0) {
          v = P.mw[m] * (K::kernel(q, q0, P.k, t...) + K::kernel(q, -q0, P.k, t...));
          if (P.T > 0 && m == 0) v += P.T * K::kernel(q, (ctype)0, P.k, t...);
        } else if constexpr (ANG == 1) {
          const ctype cs = 2 * (P.x[1][j] - (ctype)0.5);
          xw *= 2 * P.w[1][j];
          v = P.mw[m] * (K::kernel(q, cs, q0, P.k, t...) + K::kernel(q, cs, -q0, P.k, t...));
          if (P.T > 0 && m == 0) v += P.T * K::kernel(q, cs, (ctype)0, P.k, t...);
        } else {
          const ctype cs = 2 * (P.x[1][j] - (ctype)0.5);
          const ctype phi = two_pi<ctype>() * P.x[2][l];
          xw *= two_pi<ctype>() * P.w[2][l] * 2 * P.w[1][j];
          v = P.mw[m] * (K::kernel(q, cs, phi, q0, P.k, t...) + K::kernel(q, cs, phi, -q0, P.k, t...));
          if (P.T > 0 && m == 0) v += P.T * K::kernel(q, cs, phi, (ctype)0, P.k, t...);
        }
        return ie * xw * v;
      }
    };

    // Integrator{,Angle,4D}FiniteTx0GPU: explicit sum over the first ns frequencies plus a GL
    // integral on a log-mapped q0 tail (integrator_finiteTx0_gpu.hh:21-62,
    // integrator_angle_finiteTx0_gpu.hh:21-69, integrator_4D_finiteTx0_gpu.hh:21-74).
    // The tail rule is on axis 1 (radial only), 2 (with cos) or 3 (with cos and phi).
    template <int d, int ANG> struct FTx0 {
      static constexpr int TAIL = ANG == 0 ? 1 : (ANG == 1 ? 2 : 3);
      template <typename ctype> __host__ __device__ static long long points(const Params<ctype> &P)
      {
        long long p = (long long)P.n[0] * (P.ns + P.n[TAIL]);
        if (ANG >= 1) p *= P.n[1];
        if (ANG == 2) p *= P.n[2];
        return p;
      }
      template <class K, typename NT, typename ctype, class... Args>
      __device__ static NT eval(const Params<ctype> &P, long long idx, const Args &...t)
      {
        const int nz = P.ns + P.n[TAIL];
        const int m = (int)(idx % nz);
        idx /= nz;
        int l = 0, j = 0;
        if (ANG == 2) {
          l = (int)(idx % P.n[2]);
          idx /= P.n[2];
        }
        if (ANG >= 1) {
          j = (int)(idx % P.n[1]);
          idx /= P.n[1];
        }
        const int i = (int)idx;
        const ctype q = P.k * sqrt(P.x[0][i] * P.x_extent);
        const ctype base = (ANG == 2 ? (q / (ctype)2 * P.k * P.k) : S_d<ctype>(d - 1) * (powi(q, d - 3) / (ctype)2 * P.k * P.k)) *
                           (ANG == 1 ? (ctype)0.5 : (ctype)1);
        const int dd = ANG == 2 ? 4 : d;
        ctype sw = P.w[0][i] * P.x_extent;
        ctype cs = 0, phi = 0;
        if (ANG >= 1) {
          cs = 2 * (P.x[1][j] - (ctype)0.5);
          sw *= 2 * P.w[1][j];
        }
        if (ANG == 2) {
          phi = two_pi<ctype>() * P.x[2][l];
          sw *= two_pi<ctype>() * P.w[2][l];
        }
        auto Kc = [&](ctype q0) -> NT {
          if constexpr (ANG == 0)
            return K::kernel(q, q0, P.k, t...);
          else if constexpr (ANG == 1)
            return K::kernel(q, cs, q0, P.k, t...);
          else
            return K::kernel(q, cs, phi, q0, P.k, t...);
        };
        if (m < P.ns) {  // explicit sum
          const ctype ie = P.T * base / powi(two_pi<ctype>(), dd - 1);
          const ctype q0 = two_pi<ctype>() * P.T * m;
          return ie * sw * (m == 0 ? Kc((ctype)0) : Kc(q0) + Kc(-q0));
        }
        const int r = m - P.ns;  // tail integral
        const ctype q0 = P.k * (exp(P.log_start + P.log_ext * P.x[TAIL][r]) - P.off);
        const ctype ie = base * P.k / powi(two_pi<ctype>(), dd);
        const ctype wt = sw * (P.w[TAIL][r] * P.log_ext * q0 / P.k);
        return ie * wt * (Kc(q0) + Kc(-q0));
      }
    };
  } // namespace fam
} // namespace gbint
