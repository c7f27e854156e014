// test_qmc.cu -- the QMC integrators of the drop-in (include/gbint/qmc.hh) on the reference's
// own test cases (DiFfRG/tests/physics/integration/integrator_qmc.cc, integrator_angle_qmc.cc,
// integrator_4D_qmc.cc: volume integrals and random polynomials against closed forms), written
// as a user translation unit would include them.
//
// Output, one line per case: "<case> <value> <exact> <error estimate> <lattice n> <shifts m>
// <evaluations>"; tests/test_gpu_qmc.py checks them.
#include <DiFfRG/physics/integration/integrator_4D_qmc.hh>
#include <DiFfRG/physics/integration/integrator_angle_qmc.hh>
#include <DiFfRG/physics/integration/integrator_qmc.hh>

#include <cmath>
#include <cstdio>
#include <random>

using namespace DiFfRG;

namespace
{
  // q polynomial of degree 5, as the reference's PolyIntegrand
  struct Poly1 {
    static __forceinline__ __host__ __device__ double kernel(const double q, const double, const double, const double x0,
                                                             const double x1, const double x2, const double x3,
                                                             const double x4, const double x5)
    {
      return x0 + q * (x1 + q * (x2 + q * (x3 + q * (x4 + q * x5))));
    }
    static __forceinline__ __host__ __device__ double constant(const double, const double c, const double, const double,
                                                               const double, const double, const double, const double)
    {
      return c;
    }
  };
  // q polynomial x cos polynomial
  struct PolyAngle {
    static __forceinline__ __host__ __device__ double kernel(const double q, const double cs, const double,
                                                             const double, const double x0, const double x1,
                                                             const double x2, const double x3, const double c0,
                                                             const double c1, const double c2, const double c3)
    {
      return (x0 + q * (x1 + q * (x2 + q * x3))) * (c0 + cs * (c1 + cs * (c2 + cs * c3)));
    }
    static __forceinline__ __host__ __device__ double constant(const double, const double c, const double, const double,
                                                               const double, const double, const double, const double,
                                                               const double, const double)
    {
      return c;
    }
  };
  // q x cos1 x cos2 x phi polynomials (integrator_4D_qmc.cc:14-37)
  struct Poly4 {
    static __forceinline__ __host__ __device__ double kernel(const double q, const double c1, const double c2,
                                                             const double phi, const double, const double,
                                                             const double x0, const double x1, const double x2,
                                                             const double a0, const double a2, const double b0,
                                                             const double b1, const double p0, const double p1)
    {
      return (x0 + q * (x1 + q * x2)) * (a0 + a2 * c1 * c1) * (b0 + b1 * c2) * (p0 + p1 * phi);
    }
    static __forceinline__ __host__ __device__ double constant(const double, const double c, const double,
                                                               const double, const double, const double, const double,
                                                               const double, const double, const double, const double)
    {
      return c;
    }
  };

  double S_d(int d)
  {
    const double pi = M_PI;
    return d == 1 ? 2 : d == 2 ? 2 * pi : d == 3 ? 4 * pi : 2 * pi * pi;
  }
  // int_0^Q q^(d-1) sum_k a_k q^k dq
  double radial(int d, double Q, const double *a, int n)
  {
    double s = 0;
    for (int k = 0; k < n; ++k) s += a[k] * std::pow(Q, d + k) / (d + k);
    return s;
  }

  template <class I> void report(const char *tag, double v, double exact, const I &integ)
  {
    const auto st = integ.last_stats();
    std::printf("%s %.17g %.17g %.6e %llu %llu %llu\n", tag, v, exact, st.error[0], st.n, st.m, st.evaluations);
  }
} // namespace

int main()
{
  std::mt19937_64 rng(20240519);
  std::uniform_real_distribution<double> U(-1.0, 1.0), P(0.3, 1.0), X(1.0, 2.0);
  const double pi = M_PI;
  char tag[64];
  // IntegratorQMC<d>: volume integral (rel_tol 1e-6, maxeval 2e6) and random polynomials
  auto one_d = [&](auto dimc) {
    constexpr int d = decltype(dimc)::value;
    const double xe = X(rng), k = P(rng), Q = std::sqrt(xe) * k;
    IntegratorQMC<d, double, Poly1> integ(xe, 1e-6, 1e-16, 2000000);
    const double one[1] = {1.0};
    double v = integ.request(k, 0., 1., 0., 0., 0., 0., 0.).get();
    std::snprintf(tag, sizeof tag, "QMC%d_volume", d);
    report(tag, v, S_d(d) / std::pow(2 * pi, d) * radial(d, Q, one, 1), integ);
    IntegratorQMC<d, double, Poly1> integ2(xe, 1e-4, 1e-16, 500000);
    double a[6];
    for (auto &x : a) x = U(rng);
    if (d == 1) a[0] = 0;  // the reference keeps the 1D integrand regular at q = 0
    const double c = U(rng);
    v = integ2.get(k, c, a[0], a[1], a[2], a[3], a[4], a[5]);
    std::snprintf(tag, sizeof tag, "QMC%d_poly", d);
    report(tag, v, c + S_d(d) / std::pow(2 * pi, d) * radial(d, Q, a, 6), integ2);
  };
  one_d(std::integral_constant<int, 1>{});
  one_d(std::integral_constant<int, 2>{});
  one_d(std::integral_constant<int, 3>{});
  one_d(std::integral_constant<int, 4>{});
  // IntegratorAngleQMC<d>: q polynomial x cos polynomial, exact = S_d/(2pi)^d int q^(d-1) poly(q)
  // x (1/2) int_-1^1 cpoly
  auto angle = [&](auto dimc) {
    constexpr int d = decltype(dimc)::value;
    const double xe = X(rng), k = P(rng), Q = std::sqrt(xe) * k;
    IntegratorAngleQMC<d, double, PolyAngle> integ(xe, 1e-4, 1e-16, 1000000);
    double a[4], b[4];
    for (auto &x : a) x = U(rng);
    for (auto &x : b) x = U(rng);
    const double c = U(rng);
    const double v = integ.get(k, c, a[0], a[1], a[2], a[3], b[0], b[1], b[2], b[3]);
    const double ang = 0.5 * (2 * b[0] + 2.0 / 3.0 * b[2]);
    std::snprintf(tag, sizeof tag, "AngleQMC%d_poly", d);
    report(tag, v, c + S_d(d) / std::pow(2 * pi, d) * radial(d, Q, a, 4) * ang, integ);
  };
  angle(std::integral_constant<int, 2>{});
  angle(std::integral_constant<int, 3>{});
  angle(std::integral_constant<int, 4>{});
  // Integrator4DQMC (rel_tol 1e-4, maxeval 5e5): volume and random polynomials
  {
    const double xe = X(rng), k = P(rng), Q = std::sqrt(xe) * k;
    Integrator4DQMC<double, Poly4> integ(xe, 1e-4, 1e-16, 500000);
    // c + int q^3 poly dq * int sqrt(1-c1^2) (a0 + a2 c1^2) dc1 * int (b0 + b1 c2) dc2 *
    // int (p0 + p1 phi) dphi / (2 pi)^4
    auto exact = [&](double c, const double *x, double a0, double a2, double b0, double p0, double p1) {
      return c + radial(4, Q, x, 3) * ((4 * a0 + a2) * pi / 8) * (2 * b0) * (p0 * 2 * pi + p1 * 2 * pi * pi) /
                     std::pow(2 * pi, 4);
    };
    const double unit[3] = {1.0, 0.0, 0.0};
    double v = integ.get(k, 0., 1., 0., 0., 1., 0., 1., 0., 1., 0.);
    report("4DQMC_volume", v, exact(0, unit, 1, 0, 1, 1, 0), integ);  // V_4(Q) / (2 pi)^4
    double x[3], a0 = U(rng), a2 = U(rng), b0 = U(rng), b1 = U(rng), p0 = U(rng), p1 = U(rng);
    for (auto &y : x) y = U(rng);
    const double c = U(rng);
    v = integ.get(k, c, x[0], x[1], x[2], a0, a2, b0, b1, p0, p1);
    report("4DQMC_poly", v, exact(c, x, a0, a2, b0, p0, p1), integ);
  }
  return 0;
}
