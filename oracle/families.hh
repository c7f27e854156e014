// families.hh -- TEST INFRASTRUCTURE ONLY (see oracle.hh).
//
// FP64 restatement of DiFfRG's integrator families.  Every family evaluates
//     constant(k) + sum over its tensor-product quadrature of weight * KERNEL(point)
// with the maps and Jacobians of the reference's *_cpu.hh files; each function below cites
// the loop it follows.  Reference restrictions on equal angular orders are lifted: every
// angular axis has its own Gauss-Legendre rule of its own order, which coincides with the
// reference whenever the orders are equal (the reference throws or mis-indexes otherwise:
// integrator_4D_cpu.hh:83 divides by grid_sizes[2] where grid_sizes[3] is meant,
// integrator_3D_cpu.hh:39-40 throws, integrator_4D_finiteT*_cpu.hh read the phi nodes from
// the cos rule).
#pragma once

#include "oracle.hh"

#include <array>
#include <functional>
#include <map>
#include <mutex>

namespace oracle
{
  enum Family : int {
    F_1D = 1,        // IntegratorTBB<d>                    integrator_cpu.hh:50-73
    F_ANGLE = 2,     // IntegratorAngleTBB<d>               integrator_angle_cpu.hh:59-84
    F_3D = 3,        // Integrator3DTBB                     integrator_3D_cpu.hh:42-69
    F_4D2ANG = 4,    // Integrator4D2AngTBB                 integrator_4D_2ang_cpu.hh:59-94
    F_4D = 5,        // Integrator4DTBB                     integrator_4D_cpu.hh:64-98
    F_CART1 = 6,     // Integrator1DCartesianTBB            integrator_1D_cartesian_cpu.hh:121-136
    F_CART2 = 7,     // Integrator2DCartesianTBB            integrator_2D_cartesian_cpu.hh:111-131
    F_CART3 = 8,     // Integrator3DCartesianTBB            integrator_3D_cartesian_cpu.hh:97-121
    F_2DPQ0 = 9,     // Integrator2Dpq0TBB                  integrator_2Dpq0_cpu.hh:64-95
    F_2DPX0 = 10,    // Integrator2Dpx0TBB                  integrator_2Dpx0_cpu.hh:78-106
    F_3DPQ0 = 11,    // Integrator3Dpq0TBB                  integrator_3Dpq0_cpu.hh:43-75
    F_3DPX0 = 12,    // Integrator3Dpx0TBB                  integrator_3Dpx0_cpu.hh:43-75
    F_FTQ0 = 13,     // IntegratorFiniteTq0TBB<d>           integrator_finiteTq0_cpu.hh:80-113
    F_ANGLE_FTQ0 = 14, // IntegratorAngleFiniteTq0TBB<d>    integrator_angle_finiteTq0_cpu.hh:84-122
    F_4D_FTQ0 = 15,  // Integrator4DFiniteTq0TBB            integrator_4D_finiteTq0_cpu.hh:80-125
    F_FTX0 = 16,     // IntegratorFiniteTx0TBB<d>           integrator_finiteTx0_cpu.hh:64-107
    F_ANGLE_FTX0 = 17, // IntegratorAngleFiniteTx0TBB<d>    integrator_angle_finiteTx0_cpu.hh:67-122
    F_4D_FTX0 = 18,  // Integrator4DFiniteTx0TBB            integrator_4D_finiteTx0_cpu.hh:66-122
    F_CONST = 19,    // IntegratorConstant<d>               integrator_constant.hh:47-52
  };

  // Where a kernel is evaluated.  Fields a family does not use stay 0.
  struct Point {
    double q = 0, c1 = 0, c2 = 0, phi = 0, q0 = 0;  // spherical families
    double qx = 0, qy = 0, qz = 0;                 // Cartesian families
    double k = 0;
  };

  struct FamilyDesc {
    int family = F_ANGLE;
    int d = 4;                 // template dimension where the reference has one
    int n[4] = {0, 0, 0, 0};   // reference grid_sizes (finite-T: spatial orders + x0 order)
    double x_extent = 1;
    double x0_extent = 0;      // q0_extent for p{q}0, x0_extent for p{x}0 and finite-T x0
    int x0_summands = 0;
    double T = 0;
    double E = 0;              // typical energy of the Matsubara rule (already resolved)
    int mats_min = 32, mats_vacuum = 48, mats_add = 0;
    double qmin[3] = {-kPi, -kPi, -kPi};
    double qmax[3] = {kPi, kPi, kPi};
  };

  // S_d of math.hh:104-121 (surface of the unit sphere in d dimensions)
  inline double S_d(int d) { return 2.0 * std::pow(kPi, d / 2.0) / std::tgamma(d / 2.0); }
  inline double powi(double x, int n)
  {
    if (n < 0) return 1.0 / powi(x, -n);
    double r = 1;
    for (int i = 0; i < n; ++i) r *= x;
    return r;
  }

  struct RuleCache {
    std::mutex m;
    std::map<int, std::pair<std::vector<double>, std::vector<double>>> gl;
    const std::pair<std::vector<double>, std::vector<double>> &get(int n)
    {
      std::lock_guard<std::mutex> lk(m);
      auto it = gl.find(n);
      if (it != gl.end()) return it->second;
      auto &e = gl[n];
      gauss_legendre01(n, e.first, e.second);
      return e;
    }
  };
  inline RuleCache &rules()
  {
    static RuleCache rc;
    return rc;
  }

  // Evaluate one integral of family `f` for kernel `K` (callable: double(const Point&)).
  template <typename K> double integrate(const FamilyDesc &f, double k, double constant, K &&kern)
  {
    PairwiseSum acc;
    Point P;
    P.k = k;
    const double tp = 2 * kPi;
    switch (f.family) {
    case F_1D: {  // integrator_cpu.hh:59-69
      const auto &X = rules().get(f.n[0]);
      const double Sd = S_d(f.d);
      for (int i = 0; i < f.n[0]; ++i) {
        P.q = k * std::sqrt(X.first[i] * f.x_extent);
        const double ie = Sd * (powi(P.q, f.d - 2) / 2.0 * k * k) / powi(tp, f.d);
        acc.add(ie * X.second[i] * f.x_extent * kern(P));
      }
      break;
    }
    case F_ANGLE: {  // integrator_angle_cpu.hh:67-80
      const auto &X = rules().get(f.n[0]);
      const auto &A = rules().get(f.n[1]);
      const double Sd = S_d(f.d);
      for (int i = 0; i < f.n[0]; ++i) {
        P.q = k * std::sqrt(X.first[i] * f.x_extent);
        const double ie = Sd * (powi(P.q, f.d - 2) / 2.0 * k * k) * 0.5 / powi(tp, f.d);
        for (int j = 0; j < f.n[1]; ++j) {
          P.c1 = 2 * (A.first[j] - 0.5);
          const double w = 2 * A.second[j] * X.second[i] * f.x_extent;
          acc.add(ie * w * kern(P));
        }
      }
      break;
    }
    case F_3D: {  // integrator_3D_cpu.hh:49-64 (phi axis has its own order n[2])
      const auto &X = rules().get(f.n[0]);
      const auto &C = rules().get(f.n[1]);
      const auto &F = rules().get(f.n[2]);
      for (int i = 0; i < f.n[0]; ++i) {
        P.q = k * std::sqrt(X.first[i] * f.x_extent);
        const double ie = (P.q / 2.0 * k * k) / powi(tp, 3);
        for (int j = 0; j < f.n[1]; ++j) {
          P.c1 = 2 * (C.first[j] - 0.5);
          for (int l = 0; l < f.n[2]; ++l) {
            P.phi = tp * F.first[l];
            const double w = tp * F.second[l] * 2 * C.second[j] * X.second[i] * f.x_extent;
            acc.add(ie * w * kern(P));
          }
        }
      }
      break;
    }
    case F_4D2ANG: {  // integrator_4D_2ang_cpu.hh:66-90
      const auto &X = rules().get(f.n[0]);
      const auto &C1 = rules().get(f.n[1]);
      const auto &C2 = rules().get(f.n[2]);
      for (int i = 0; i < f.n[0]; ++i) {
        P.q = k * std::sqrt(X.first[i] * f.x_extent);
        for (int j = 0; j < f.n[1]; ++j) {
          P.c1 = 2 * (C1.first[j] - 0.5);
          const double ie = tp * (P.q * P.q * 0.5 * k * k) * std::sqrt(1.0 - P.c1 * P.c1) / powi(tp, 4);
          for (int l = 0; l < f.n[2]; ++l) {
            P.c2 = 2 * (C2.first[l] - 0.5);
            const double w = 2 * C2.second[l] * 2 * C1.second[j] * X.second[i] * f.x_extent;
            acc.add(ie * w * kern(P));
          }
        }
      }
      break;
    }
    case F_4D: {  // integrator_4D_cpu.hh:71-96 with cos2 index = z / n3, phi index = z % n3
      const auto &X = rules().get(f.n[0]);
      const auto &C1 = rules().get(f.n[1]);
      const auto &C2 = rules().get(f.n[2]);
      const auto &F = rules().get(f.n[3]);
      for (int i = 0; i < f.n[0]; ++i) {
        P.q = k * std::sqrt(X.first[i] * f.x_extent);
        for (int j = 0; j < f.n[1]; ++j) {
          P.c1 = 2 * (C1.first[j] - 0.5);
          const double ie = (P.q * P.q * 0.5 * k * k) * std::sqrt(1.0 - P.c1 * P.c1) / powi(tp, 4);
          for (int l = 0; l < f.n[2]; ++l) {
            P.c2 = 2 * (C2.first[l] - 0.5);
            for (int m = 0; m < f.n[3]; ++m) {
              P.phi = tp * F.first[m];
              const double w =
                  tp * F.second[m] * 2 * C2.second[l] * 2 * C1.second[j] * X.second[i] * f.x_extent;
              acc.add(ie * w * kern(P));
            }
          }
        }
      }
      break;
    }
    case F_CART1:
    case F_CART2:
    case F_CART3: {  // integrator_{1,2,3}D_cartesian_cpu.hh: q = qmin + ext*t, w = ext*w_t, /(2pi)^d
      const int dim = f.family - F_CART1 + 1;
      const double ie = powi(tp, -dim);
      const auto &Rx = rules().get(f.n[0]);
      const auto &Ry = rules().get(dim > 1 ? f.n[1] : 1);
      const auto &Rz = rules().get(dim > 2 ? f.n[2] : 1);
      const double ex = f.qmax[0] - f.qmin[0], ey = f.qmax[1] - f.qmin[1], ez = f.qmax[2] - f.qmin[2];
      const int ny = dim > 1 ? f.n[1] : 1, nz = dim > 2 ? f.n[2] : 1;
      for (int i = 0; i < f.n[0]; ++i) {
        P.qx = f.qmin[0] + ex * Rx.first[i];
        for (int j = 0; j < ny; ++j) {
          if (dim > 1) P.qy = f.qmin[1] + ey * Ry.first[j];
          for (int l = 0; l < nz; ++l) {
            if (dim > 2) P.qz = f.qmin[2] + ez * Rz.first[l];
            double w = ex * Rx.second[i];
            if (dim > 1) w *= ey * Ry.second[j];
            if (dim > 2) w *= ez * Rz.second[l];
            acc.add(ie * w * kern(P));
          }
        }
      }
      break;
    }
    case F_2DPQ0:
    case F_2DPX0: {  // integrator_2Dpq0_gpu.hh:33-46 / integrator_2Dpx0_cpu.hh:88-101
      // int_element = (1/2 k^2) S_2 (1/2) [* k for px0] / (2pi)^3.  The GPU kernel of 2Dpq0 and
      // the analytic test (tests/physics/integration/integrator_2Dpq0_cpu.cc:96-98) carry the
      // S_2/2 factor that integrator_2Dpq0_cpu.hh:78-81 declares but never multiplies in; the
      // GPU/analytic form is the one restated here.
      const bool px = f.family == F_2DPX0;
      const auto &X = rules().get(f.n[0]);
      const auto &C = rules().get(f.n[1]);
      const auto &Q = rules().get(f.n[2]);
      for (int i = 0; i < f.n[0]; ++i) {
        P.q = k * std::sqrt(X.first[i] * f.x_extent);
        const double ie = (0.5 * k * k) * tp * 0.5 * (px ? k : 1.0) / powi(tp, 3);
        for (int j = 0; j < f.n[1]; ++j) {
          P.c1 = 2 * (C.first[j] - 0.5);
          for (int l = 0; l < f.n[2]; ++l) {
            const double q0 = px ? k * Q.first[l] * f.x0_extent : Q.first[l] * f.x0_extent;
            const double w = Q.second[l] * f.x0_extent * 2 * C.second[j] * X.second[i] * f.x_extent;
            P.q0 = q0;
            double v = kern(P);
            P.q0 = -q0;
            v += kern(P);
            acc.add(ie * w * v);
          }
        }
      }
      break;
    }
    case F_3DPQ0:
    case F_3DPX0: {  // integrator_3Dp{q,x}0_cpu.hh:54-70; phi axis n[2], q0 axis n[3]
      // px0 carries the extra k of x0 = q0/k (integrator_3Dpx0_cpu.hh:57-59)
      const bool px = f.family == F_3DPX0;
      const auto &X = rules().get(f.n[0]);
      const auto &C = rules().get(f.n[1]);
      const auto &F = rules().get(f.n[2]);
      const auto &Q = rules().get(f.n[3]);
      for (int i = 0; i < f.n[0]; ++i) {
        P.q = k * std::sqrt(X.first[i] * f.x_extent);
        const double ie = (P.q / 2.0 * k * k) * (px ? k : 1.0) / powi(tp, 4);
        for (int j = 0; j < f.n[1]; ++j) {
          P.c1 = 2 * (C.first[j] - 0.5);
          for (int l = 0; l < f.n[2]; ++l) {
            P.phi = tp * F.first[l];
            for (int m = 0; m < f.n[3]; ++m) {
              const double q0 = px ? k * Q.first[m] * f.x0_extent : Q.first[m] * f.x0_extent;
              const double w =
                  Q.second[m] * f.x0_extent * tp * F.second[l] * 2 * C.second[j] * X.second[i] * f.x_extent;
              P.q0 = q0;
              double v = kern(P);
              P.q0 = -q0;
              v += kern(P);
              acc.add(ie * w * v);
            }
          }
        }
      }
      break;
    }
    case F_FTQ0:
    case F_ANGLE_FTQ0:
    case F_4D_FTQ0: {  // integrator_{,angle_,4D_}finiteTq0_cpu.hh: T f(0) + sum_i w_i [f(x_i)+f(-x_i)]
      const MatsubaraRule M = provider_matsubara(f.T, f.E, f.mats_min, f.mats_vacuum, f.mats_add);
      const auto &X = rules().get(f.n[0]);
      const int fam = f.family;
      const int d = fam == F_4D_FTQ0 ? 4 : f.d;
      const int nc = fam == F_FTQ0 ? 1 : f.n[1];
      const int nf = fam == F_4D_FTQ0 ? f.n[2] : 1;
      const auto &C = rules().get(nc);
      const auto &F = rules().get(nf);
      for (int i = 0; i < f.n[0]; ++i) {
        P.q = k * std::sqrt(X.first[i] * f.x_extent);
        double ie;
        if (fam == F_FTQ0)
          ie = S_d(d - 1) * (powi(P.q, d - 3) / 2.0 * k * k) / powi(tp, d - 1);
        else if (fam == F_ANGLE_FTQ0)
          ie = S_d(d - 1) * (powi(P.q, d - 3) / 2.0 * k * k) * 0.5 / powi(tp, d - 1);
        else
          ie = (powi(P.q, d - 3) / 2.0 * k * k) / powi(tp, d - 1);
        for (int j = 0; j < nc; ++j) {
          if (fam != F_FTQ0) P.c1 = 2 * (C.first[j] - 0.5);
          for (int l = 0; l < nf; ++l) {
            if (fam == F_4D_FTQ0) P.phi = tp * F.first[l];
            double xw = X.second[i] * f.x_extent;
            if (fam == F_ANGLE_FTQ0) xw *= 2 * C.second[j];
            if (fam == F_4D_FTQ0) xw *= tp * F.second[l] * 2 * C.second[j];
            for (size_t m = 0; m < M.x.size(); ++m) {
              const double w = xw * M.w[m];
              P.q0 = M.x[m];
              double v = kern(P);
              P.q0 = -M.x[m];
              v += kern(P);
              acc.add(ie * w * v);
              // the integrator's own m_T decides (also when the rule fell back to the vacuum
              // form for E/T > 100), as in integrator_finiteTq0_cpu.hh:107-108
              if (f.T > 0 && m == 0) {
                P.q0 = 0;
                acc.add(ie * xw * f.T * kern(P));
              }
            }
          }
        }
      }
      break;
    }
    case F_FTX0:
    case F_ANGLE_FTX0:
    case F_4D_FTX0: {  // integrator_{,angle_,4D_}finiteTx0_cpu.hh: explicit sum + log-mapped GL tail
      const int fam = f.family;
      const int d = fam == F_4D_FTX0 ? 4 : f.d;
      // grid: spatial orders, then n_x0 = tail order; summands per set_T (:41-50)
      const bool Tzero = std::fabs(f.T) <= 1e-12;
      const int ns = Tzero ? 0 : f.x0_summands;
      const int nx0 = (fam == F_FTX0 ? f.n[1] : fam == F_ANGLE_FTX0 ? f.n[2] : f.n[3]) + f.x0_summands - ns;
      const auto &X = rules().get(f.n[0]);
      const int nc = fam == F_FTX0 ? 1 : f.n[1];
      const int nf = fam == F_4D_FTX0 ? f.n[2] : 1;
      const auto &C = rules().get(nc);
      const auto &F = rules().get(nf);
      const auto &Q = rules().get(nx0);
      const double mT = Tzero ? 0.0 : f.T;
      const double start = (2 * ns * kPi * mT) / k;
      const double off = Tzero ? 1e-3 : 0.0;
      const double log_start = std::log(start + off);
      const double log_ext = std::log(f.x0_extent / (start + off));
      const double Sdm1 = S_d(d - 1);
      for (int i = 0; i < f.n[0]; ++i) {
        P.q = k * std::sqrt(X.first[i] * f.x_extent);
        double ie_int, ie_sum;
        if (fam == F_FTX0) {
          ie_int = Sdm1 * (powi(P.q, d - 3) / 2.0 * k * k) * k / powi(tp, d);
          ie_sum = mT * Sdm1 * (powi(P.q, d - 3) / 2.0 * k * k) / powi(tp, d - 1);
        } else if (fam == F_ANGLE_FTX0) {
          ie_int = Sdm1 * (powi(P.q, d - 3) / 2.0 * k * k) * k * 0.5 / powi(tp, d);
          ie_sum = mT * Sdm1 * (powi(P.q, d - 3) / 2.0 * k * k) * 0.5 / powi(tp, d - 1);
        } else {
          ie_int = (powi(P.q, d - 3) / 2.0 * k * k) * k / powi(tp, d);
          ie_sum = mT * (powi(P.q, d - 3) / 2.0 * k * k) / powi(tp, d - 1);
        }
        for (int j = 0; j < nc; ++j) {
          if (fam != F_FTX0) P.c1 = 2 * (C.first[j] - 0.5);
          for (int l = 0; l < nf; ++l) {
            if (fam == F_4D_FTX0) P.phi = tp * F.first[l];
            double sw = X.second[i] * f.x_extent;
            if (fam == F_ANGLE_FTX0) sw *= 2 * C.second[j];
            if (fam == F_4D_FTX0) sw *= tp * F.second[l] * 2 * C.second[j];
            for (int m = 0; m < nx0; ++m) {  // log-mapped tail integral
              const double q0 = k * (std::exp(log_start + log_ext * Q.first[m]) - off);
              const double w = sw * (Q.second[m] * log_ext * q0 / k);
              P.q0 = q0;
              double v = kern(P);
              P.q0 = -q0;
              v += kern(P);
              acc.add(ie_int * w * v);
            }
            for (int m = 0; m < ns; ++m) {  // explicit Matsubara sum
              const double q0 = tp * mT * m;
              double v;
              if (m == 0) {
                P.q0 = 0;
                v = kern(P);
              } else {
                P.q0 = q0;
                v = kern(P);
                P.q0 = -q0;
                v += kern(P);
              }
              acc.add(ie_sum * sw * v);
            }
          }
        }
      }
      break;
    }
    case F_CONST: {  // integrator_constant.hh:51: constant + kernel(k) * S_d / (2 pi)^d
      acc.add(kern(P) * S_d(f.d) / powi(tp, f.d));
      break;
    }
    default:
      throw std::invalid_argument("unknown family");
    }
    return constant + acc.total();
  }
} // namespace oracle
