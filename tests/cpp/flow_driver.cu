// flow_driver.cu -- runs one flow class in the form DiFfRG's code generator writes it (a
// flows/<dir>/<X>.cu file with its X.hh, X.kernel and the example's def.hh, compiled UNCHANGED
// against the drop-in headers) through the GB300 integrators, and checks every value against
// the FP64 oracle (oracle/families.hh: the restatement of the reference's CPU integrators)
// evaluating the same KERNEL class on the host over the same quadrature.
//
// Build (tests/test_gpu_flows.py does this):
//   nvcc -std=c++20 --expt-relaxed-constexpr -I include/gbint/compat -I include -I oracle
//        -I <example dir> -DGBINT_FLOW_SOURCE='"flows/AA/ZA.cu"' -DGBINT_FLOW_NAME=ZA
//        -DGBINT_FLOW_KIND=1 -DGBINT_FLOW_FAMILY=2 flow_driver.cu -lgbint
// Kinds (the two call signatures of the reference's examples):
//   1  get/request(k, p, 7 x TexLinearInterpolator1D<double, LogarithmicCoordinates1D<float>>, m2)
//      -- Examples/YangMills/SP/flows/*/ (IntegratorAngle, Integrator4D2Ang, Integrator4D)
//   2  get/request<double | autodiff::real>(k, N, T, rhoPhi, m2Pi, m2Sigma)
//      -- Examples/ONfiniteT/flows/V (IntegratorTBB<3>), value and m2Pi-derivative
// GBINT_FLOW_FAMILY is the oracle's family id (2 angle, 4 4D2Ang, 5 4D, 1 radial).
// Output: one line per value "<tag> gpu host abs_host rel_err" and a final "MAX rel_err";
// exit status 0 when every value agrees to GBINT_FLOW_TOL (default 1e-12) relative to the
// host integral of |integrand| (the scale on which the FP64 sums are accurate).
#include <array>
#include <cmath>
#include <cstdio>
#include <string>
#include <tuple>
#include <vector>

#include GBINT_FLOW_SOURCE

#include "families.hh"  // the oracle (test infrastructure)

#ifndef GBINT_FLOW_TOL
#define GBINT_FLOW_TOL 1e-12
#endif

#define GBINT_CAT2(a, b) a##b
#define GBINT_CAT(a, b) GBINT_CAT2(a, b)
using FlowClass = DiFfRG::Flows::GBINT_CAT(GBINT_FLOW_NAME, _integrator);
using KernelClass = GBINT_CAT(GBINT_FLOW_NAME, _kernel)<__REGULATOR__>;

namespace
{
  // component c of a result (value 0, derivative 1)
  inline double comp(double v, int) { return v; }
  template <typename T> double comp(const gbint::dual<T> &v, int c) { return c ? (double)v.d : (double)v.v; }

  // the KERNEL at an oracle point, with the family's coordinate list
  template <int FAM, class... A> auto kernel_at(const oracle::Point &P, const A &...a)
  {
    if constexpr (FAM == oracle::F_1D)
      return KernelClass::kernel(P.q, P.k, a...);
    else if constexpr (FAM == oracle::F_ANGLE)
      return KernelClass::kernel(P.q, P.c1, P.k, a...);
    else if constexpr (FAM == oracle::F_4D2ANG)
      return KernelClass::kernel(P.q, P.c1, P.c2, P.k, a...);
    else if constexpr (FAM == oracle::F_3D)
      return KernelClass::kernel(P.q, P.c1, P.phi, P.k, a...);
    else
      return KernelClass::kernel(P.q, P.c1, P.c2, P.phi, P.k, a...);
  }

  // oracle integral of component c of the KERNEL (and of its modulus)
  template <class... A>
  std::pair<double, double> host_integral(const oracle::FamilyDesc &f, double k, int c, const A &...a)
  {
    const double cst = comp(KernelClass::constant(k, a...), c);
    const double v = oracle::integrate(f, k, cst, [&](const oracle::Point &P) {
      return comp(kernel_at<GBINT_FLOW_FAMILY>(P, a...), c);
    });
    const double s = oracle::integrate(f, k, std::fabs(cst), [&](const oracle::Point &P) {
      return std::fabs(comp(kernel_at<GBINT_FLOW_FAMILY>(P, a...), c));
    });
    return {v, s};
  }

  double g_max = 0;
  int g_bad = 0;
  void report(const char *tag, int i, double gpu, std::pair<double, double> host)
  {
    const double scale = host.second > 0 ? host.second : 1.0;
    const double err = std::fabs(gpu - host.first) / scale;
    g_max = std::fmax(g_max, err);
    if (!(err <= GBINT_FLOW_TOL)) ++g_bad;
    std::printf("%s %d %.17g %.17g %.17g %.3e\n", tag, i, gpu, host.first, host.second, err);
  }

  // seeded smooth table values base + amp * (5-point average of a uniform sequence)
  std::vector<double> seeded_values(unsigned n, unsigned seed, double base, double amp)
  {
    std::vector<double> u(n), out(n);
    unsigned long long s = 0x9E3779B97F4A7C15ull * (seed + 1);
    for (unsigned i = 0; i < n; ++i) {
      s ^= s >> 12;
      s ^= s << 25;
      s ^= s >> 27;
      u[i] = (double)((s * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
    }
    for (unsigned i = 0; i < n; ++i) {
      double acc = 0;
      int cnt = 0;
      for (int j = (int)i - 2; j <= (int)i + 2; ++j)
        if (j >= 0 && j < (int)n) {
          acc += u[j];
          ++cnt;
        }
      out[i] = base + amp * acc / cnt;
    }
    return out;
  }

  DiFfRG::JSONValue settings()
  {
    return DiFfRG::JSONValue(std::string(R"({"integration": {"x_quadrature_order": 32,
        "angle_quadrature_order": 8, "x0_quadrature_order": 16, "x0_summands": 8,
        "q0_quadrature_order": 16, "q0_summands": 8, "jacobian_quadrature_factor": 1.5,
        "cudathreadsperblock": 256, "x_extent_tolerance": 1e-3, "x0_extent_tolerance": 1e-3,
        "q0_extent_tolerance": 1e-3, "min_matsubara_size": 16, "vacuum_quad_size": 48},
        "physical": {"T": 0.1}, "output": {"verbosity": 0}})"));
  }
} // namespace

int main()
{
  using namespace DiFfRG;
  const JSONValue json = settings();
  QuadratureProvider qp(json);
  oracle::FamilyDesc f;
  f.family = GBINT_FLOW_FAMILY;
  const double x_extent = 3.0;
  f.x_extent = x_extent;

#if GBINT_FLOW_KIND == 1
  // grid orders per family (kept moderate: the host evaluates the full KERNEL at every point)
  constexpr int NAX = GBINT_FLOW_FAMILY == oracle::F_ANGLE ? 2 : (GBINT_FLOW_FAMILY == oracle::F_4D ? 4 : 3);
  constexpr std::array<uint, 4> orders = NAX == 2 ? std::array<uint, 4>{{48, 24, 0, 0}}
                                         : (NAX == 3 ? std::array<uint, 4>{{32, 12, 10, 0}}
                                                     : std::array<uint, 4>{{24, 10, 8, 6}});
  std::array<uint, NAX> gs{};
  for (int a = 0; a < NAX; ++a) gs[a] = orders[a];
  f.d = 4;
  for (int a = 0; a < NAX; ++a) f.n[a] = (int)gs[a];
  FlowClass flow(qp, gs, x_extent, json);

  using Tab = TexLinearInterpolator1D<double, LogarithmicCoordinates1D<float>>;
  const LogarithmicCoordinates1D<float> coords(64, 1e-3f, 40.f, 5.f);
  std::vector<Tab> T;
  const double base[7] = {1.0, 0.8, 1.2, 0.05, 1.0, -0.1, 1.1}, amp[7] = {0.6, 0.5, 0.4, 0.1, 0.5, 0.2, 0.5};
  for (int t = 0; t < 7; ++t) T.emplace_back(seeded_values(64, 11 + t, base[t], amp[t]), coords);
  const double k = 1.2, m2 = 0.15;
  const int NP = 32;
  std::vector<double> gpu(NP), req(NP);
  std::vector<std::future<double>> fut;
  for (int i = 0; i < NP; ++i) {
    const double p = 1e-2 * std::pow(1e3, i / (NP - 1.0));
    fut.push_back(flow.template request<double>(k, p, T[0], T[1], T[2], T[3], T[4], T[5], T[6], m2));
  }
  for (int i = 0; i < NP; ++i) {
    const double p = 1e-2 * std::pow(1e3, i / (NP - 1.0));
    gpu[i] = flow.template get<double>(k, p, T[0], T[1], T[2], T[3], T[4], T[5], T[6], m2);
    req[i] = fut[i].get();
    const auto host = host_integral(f, k, 0, p, T[0], T[1], T[2], T[3], T[4], T[5], T[6], m2);
    report("GET", i, gpu[i], host);
    report("REQUEST", i, req[i], host);
  }
#elif GBINT_FLOW_KIND == 2
  std::array<uint, 1> gs{{64}};
  f.d = 3;
  f.n[0] = 64;
  FlowClass flow(qp, gs, x_extent, json);
  const double N = 4, rhoPhi = 0.02, m2Sigma = 0.4;
  const double Ts[3] = {0.0, 0.1, 0.5};
  int idx = 0;
  for (double Temp : Ts)
    for (double k : {0.5, 1.0, 2.0}) {
      const double m2Pi = 0.05 + 0.1 * idx;
      const double v = flow.template get<double>(k, N, Temp, rhoPhi, m2Pi, m2Sigma);
      const autodiff::real mp = gbint::seed(m2Pi);
      const autodiff::real ad = flow.template get<autodiff::real>(k, N, Temp, rhoPhi, mp, (autodiff::real)m2Sigma);
      const double r = flow.template request<double>(k, N, Temp, rhoPhi, m2Pi, m2Sigma).get();
      report("GET", idx, v, host_integral(f, k, 0, N, Temp, rhoPhi, m2Pi, m2Sigma));
      report("REQUEST", idx, r, host_integral(f, k, 0, N, Temp, rhoPhi, m2Pi, m2Sigma));
      // the autodiff integrator runs on the jacobian rule (jacobian_quadrature_factor x order)
      oracle::FamilyDesc fj = f;
      fj.n[0] = (int)(1.5 * 64);
      report("AD_VALUE", idx, autodiff::val(ad), host_integral(fj, k, 0, N, Temp, rhoPhi, mp, (autodiff::real)m2Sigma));
      report("AD_DERIV", idx, autodiff::derivative(ad),
             host_integral(fj, k, 1, N, Temp, rhoPhi, mp, (autodiff::real)m2Sigma));
      ++idx;
    }
#else
#error "GBINT_FLOW_KIND must be 1 or 2"
#endif
  std::printf("MAX %.3e BAD %d\n", g_max, g_bad);
  return g_bad ? 1 : 0;
}
