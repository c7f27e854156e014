// Test driver of the host loop integrals and flow-equation bases (include/gbint/loop_integrals.hh,
// include/gbint/flow_equations.hh), compiled with g++ alone (no CUDA).
//
// Cases come on stdin, one per line; each prints one line:
//   gl n                       -> the n nodes, then the n weights of QGauss<1>(n) (17 digits)
//   li FN nt d nx ncos nm x_extent k m_extent m_order T zeta a0..a7 c0..c3 b0..b3 e0..e3
//                              -> "re im" of LoopIntegrals::FN with the integrand
//        P(q2) C(cos) [Q(q0) | Z(q0)] (integrate .. sum), P(q2) C(cos) D(cos2) F(phi) (angles):
//        P = sum a_i q2^i, C = sum c_i cos^i, Q = D = sum b_i t^i, F = sum e_i phi^i and, when
//        zeta > 0, Z(q0) = 1 at q0 = 0 else (|q0| / (2 pi T))^-zeta (the Matsubara-sum integrand
//        of DiFfRG/tests/physics/test_loop_integrals.cc:228-232); nt 1 multiplies by (1 + 0.5 i)
//        and sums in std::complex<double>.  FN: integrate angle two_angle three_angle sii saii sis
//        sais sum (sii/saii/sis/sais = spatial_[angle_]integrate_and_{integrate,sum}).
//   fe x_order angle_order jac_factor x_tol FX
//                              -> "x_extent" of a FlowEquations, or "throw <message>"
//   fet x_order angle_order jac_factor x_tol x0_order x0_tol x0_summands q0_order q0_tol q0_summands T FX FX0 FQ0
//                              -> "x_extent x0_extent q0_extent" of a FlowEquationsFiniteT
//   fe ... FX print / fet ... FQ0 print
//                              -> the print_parameters log with '|' for the newlines
//   jac x_order angle_order jac_factor x_tol FX k
//                              -> "a b": FlowEquations::integrate<AD,4>(FX) for a result type AD
//        marked for the jacobian rules, and LoopIntegrals::integrate<double,4> over
//        QGauss<1>(jac_factor * x_order) at the fitted x_extent
// Functions FX: gauss exp(-q2), rational 1/(1+q2)^4, zero (1-q2) for q2 < 1 else 0, grow exp(q2);
// FX0, FQ0 (called with signed frequencies): gauss0 exp(-q0^2), rational0 1/(1+q0^2)^4.
#include <cmath>
#include <complex>
#include <cstdio>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "gbint/flow_equations.hh"

namespace
{
  using cplx = std::complex<double>;
  constexpr double kPi = 3.141592653589793238462643383279502884;

  double poly(const std::vector<double> &c, double t)
  {
    double r = 0;
    for (size_t i = c.size(); i-- > 0;) r = r * t + c[i];
    return r;
  }

  struct Case {
    std::string fn;
    int nt = 0, d = 4, nx = 0, ncos = 0, nm = 0, m_order = 0;
    double x_extent = 1, k = 1, m_extent = 1, T = 0, zeta = 0;
    std::vector<double> a, c, b, e;
  };

  template <typename NT> NT scale(double v, int nt)
  {
    if constexpr (std::is_same_v<NT, cplx>)
      return nt ? cplx(v, 0.5 * v) : cplx(v, 0.);
    else
      return v;
  }

  template <typename NT> NT run_li(const Case &cs)
  {
    using namespace DiFfRG;
    const QGauss<1> xq(cs.nx > 0 ? cs.nx : 1);
    const QGauss<1> cq(cs.ncos > 0 ? cs.ncos : 1);
    const QGauss<1> mq(cs.nm > 0 ? cs.nm : 1);
    const double T = cs.T, zeta = cs.zeta;
    auto Zq = [&](double q0) {
      if (zeta > 0)
        return std::fabs(q0) <= std::numeric_limits<double>::epsilon() ? 1.
                                                                        : 1. / std::pow(std::fabs(q0) / (2. * kPi * T), zeta);
      return poly(cs.b, q0);
    };
    auto f1 = [&](double q2) { return scale<NT>(poly(cs.a, q2), cs.nt); };
    auto f2 = [&](double q2, double c) { return scale<NT>(poly(cs.a, q2) * poly(cs.c, c), cs.nt); };
    auto fq = [&](double q2, double q0) { return scale<NT>(poly(cs.a, q2) * Zq(q0), cs.nt); };
    auto fcq = [&](double q2, double c, double q0) {
      return scale<NT>(poly(cs.a, q2) * poly(cs.c, c) * Zq(q0), cs.nt);
    };
    auto f3 = [&](double q2, double c, double phi) {
      return scale<NT>(poly(cs.a, q2) * poly(cs.c, c) * poly(cs.e, phi), cs.nt);
    };
    auto f4 = [&](double q2, double c1, double c2, double phi) {
      return scale<NT>(poly(cs.a, q2) * poly(cs.c, c1) * poly(cs.b, c2) * poly(cs.e, phi), cs.nt);
    };
    auto fs = [&](double q0) { return scale<NT>(Zq(q0), cs.nt); };
    switch (cs.d) {
#define GBINT_LI_CASE(D)                                                                                         \
  case D:                                                                                                        \
    if (cs.fn == "integrate") return LoopIntegrals::integrate<NT, D>(f1, xq, cs.x_extent, cs.k);                 \
    if constexpr (D > 1)                                                                                         \
      if (cs.fn == "angle") return LoopIntegrals::angle_integrate<NT, D>(f2, xq, cs.x_extent, cs.k, cq);       \
    if constexpr (D > 2)                                                                                         \
      if (cs.fn == "two_angle") return LoopIntegrals::two_angle_integrate<NT, D>(f3, xq, cs.x_extent, cs.k, cq); \
    if constexpr (D > 3)                                                                                         \
      if (cs.fn == "three_angle")                                                                                \
        return LoopIntegrals::three_angle_integrate<NT, D>(f4, xq, cs.x_extent, cs.k, cq);                       \
    if (cs.fn == "sii")                                                                                          \
      return LoopIntegrals::spatial_integrate_and_integrate<NT, D>(fq, xq, cs.x_extent, cs.k, mq, cs.m_extent);  \
    if (cs.fn == "saii")                                                                                         \
      return LoopIntegrals::spatial_angle_integrate_and_integrate<NT, D>(fcq, xq, cs.x_extent, cs.k, cq, mq,     \
                                                                         cs.m_extent);                           \
    if (cs.fn == "sis")                                                                                          \
      return LoopIntegrals::spatial_integrate_and_sum<NT, D>(fq, xq, cs.x_extent, cs.k, cs.m_order, mq,         \
                                                             cs.m_extent, T);                                    \
    if (cs.fn == "sais")                                                                                         \
      return LoopIntegrals::spatial_angle_integrate_and_sum<NT, D>(fcq, xq, cs.x_extent, cs.k, cq, cs.m_order,  \
                                                                   mq, cs.m_extent, T);                          \
    break;
      GBINT_LI_CASE(1)
      GBINT_LI_CASE(2)
      GBINT_LI_CASE(3)
      GBINT_LI_CASE(4)
      GBINT_LI_CASE(5)
      GBINT_LI_CASE(6)
#undef GBINT_LI_CASE
    default:
      break;
    }
    if (cs.fn == "sum") return LoopIntegrals::sum<NT>(fs, cs.m_order, mq, cs.m_extent, T);
    throw std::invalid_argument("unknown loop integral " + cs.fn + " in d = " + std::to_string(cs.d));
  }

  std::function<double(double)> named(const std::string &name)
  {
    if (name == "gauss") return [](double q2) { return std::exp(-q2); };
    if (name == "rational") return [](double q2) { return 1. / std::pow(1. + q2, 4); };
    if (name == "zero") return [](double q2) { return q2 < 1. ? 1. - q2 : 0.; };
    if (name == "grow") return [](double q2) { return std::exp(q2); };
    // even functions of a frequency q0, for the x0 and q0 fits
    if (name == "gauss0") return [](double q0) { return std::exp(-q0 * q0); };
    if (name == "rational0") return [](double q0) { return 1. / std::pow(1. + q0 * q0, 4); };
    throw std::invalid_argument("unknown function " + name);
  }

  // DiFfRG's JSONValue accessors over a flat map of paths
  struct Json {
    std::map<std::string, double> v;
    unsigned get_uint(const std::string &p) const { return (unsigned)at(p); }
    double get_double(const std::string &p) const { return at(p); }
    int get_int(const std::string &p) const { return (int)at(p); }
    double at(const std::string &p) const
    {
      auto it = v.find(p);
      if (it == v.end()) throw std::runtime_error("missing JSON entry " + p);
      return it->second;
    }
  };

  struct Flow : DiFfRG::FlowEquations {
    Flow(const Json &j, std::function<double(double)> f) : FlowEquations(j, f) {}
    double xe() const { return x_extent; }
    unsigned jac_order() const { return jac_x_quadrature_order; }
  };
  struct FlowT : DiFfRG::FlowEquationsFiniteT {
    FlowT(const Json &j, double T, std::function<double(double)> f, std::function<double(double)> f0,
          std::function<double(double)> fq0)
        : FlowEquationsFiniteT(j, T, f, f0, fq0)
    {
    }
    double xe() const { return x_extent; }
    double x0e() const { return x0_extent; }
    double q0e() const { return q0_extent; }
  };

  // a result type that flows integrate over the jacobian rules
  struct AD {
    double v = 0;
    AD() = default;
    AD(double x) : v(x) {}
    AD &operator+=(const AD &o)
    {
      v += o.v;
      return *this;
    }
  };
  inline AD operator*(double a, const AD &b) { return AD(a * b.v); }
  inline AD operator+(const AD &a, const AD &b) { return AD(a.v + b.v); }
} // namespace

namespace DiFfRG::gbint_detail
{
  template <> struct uses_jacobian_quadrature<AD> : std::true_type {};
} // namespace DiFfRG::gbint_detail

int main()
{
  std::string line;
  while (std::getline(std::cin, line)) {
    if (line.empty()) continue;
    std::istringstream in(line);
    std::string mode;
    in >> mode;
    try {
      if (mode == "gl") {
        int n;
        in >> n;
        const DiFfRG::QGauss<1> q(n);
        for (int i = 0; i < n; ++i) std::printf("%.17g ", q.get_points()[i][0]);
        for (int i = 0; i < n; ++i) std::printf("%.17g ", q.get_weights()[i]);
        std::printf("\n");
      } else if (mode == "li") {
        Case cs;
        in >> cs.fn >> cs.nt >> cs.d >> cs.nx >> cs.ncos >> cs.nm >> cs.x_extent >> cs.k >> cs.m_extent >>
            cs.m_order >> cs.T >> cs.zeta;
        cs.a.resize(8);
        cs.c.resize(4);
        cs.b.resize(4);
        cs.e.resize(4);
        for (auto &x : cs.a) in >> x;
        for (auto &x : cs.c) in >> x;
        for (auto &x : cs.b) in >> x;
        for (auto &x : cs.e) in >> x;
        const cplx r = cs.nt ? run_li<cplx>(cs) : cplx(run_li<double>(cs), 0.);
        std::printf("%.17g %.17g\n", r.real(), r.imag());
      } else if (mode == "fe" || mode == "jac") {
        Json j;
        double xo, ao, jf, tol;
        std::string fx;
        in >> xo >> ao >> jf >> tol >> fx;
        j.v = {{"/integration/x_quadrature_order", xo}, {"/integration/angle_quadrature_order", ao},
               {"/integration/jacobian_quadrature_factor", jf}, {"/integration/x_extent_tolerance", tol},
               {"/output/verbosity", 0}};
        Flow flow(j, named(fx));
        std::string extra;
        if (mode == "fe" && (in >> extra) && extra == "print") {  // the parameter log, '|' for newlines
          std::ostringstream log;
          flow.print_parameters("log", log);
          std::string t = log.str();
          for (char &c : t)
            if (c == '\n') c = '|';
          std::printf("%s\n", t.c_str());
        } else if (mode == "fe") {
          std::printf("%.17g\n", flow.xe());
        } else {
          double k;
          in >> k;
          flow.set_k(k);
          auto f = named(fx);
          const AD a = flow.integrate<AD, 4>([&](double q2) { return AD(f(q2)); });
          const double b = DiFfRG::LoopIntegrals::integrate<double, 4>(f, DiFfRG::QGauss<1>(flow.jac_order()),
                                                                        flow.xe(), k);
          std::printf("%.17g %.17g\n", a.v, b);
        }
      } else if (mode == "fet") {
        Json j;
        double xo, ao, jf, xt, x0o, x0t, x0s, q0o, q0t, q0s, T;
        std::string fx, fx0, fq0;
        in >> xo >> ao >> jf >> xt >> x0o >> x0t >> x0s >> q0o >> q0t >> q0s >> T >> fx >> fx0 >> fq0;
        j.v = {{"/integration/x_quadrature_order", xo},     {"/integration/angle_quadrature_order", ao},
               {"/integration/jacobian_quadrature_factor", jf}, {"/integration/x_extent_tolerance", xt},
               {"/integration/x0_quadrature_order", x0o},   {"/integration/x0_extent_tolerance", x0t},
               {"/integration/x0_summands", x0s},           {"/integration/q0_quadrature_order", q0o},
               {"/integration/q0_extent_tolerance", q0t},   {"/integration/q0_summands", q0s},
               {"/output/verbosity", 0}};
        FlowT flow(j, T, named(fx), named(fx0), named(fq0));
        std::string extra;
        if ((in >> extra) && extra == "print") {
          std::ostringstream log;
          flow.print_parameters("log", log);
          std::string t = log.str();
          for (char &c : t)
            if (c == '\n') c = '|';
          std::printf("%s\n", t.c_str());
        } else
          std::printf("%.17g %.17g %.17g\n", flow.xe(), flow.x0e(), flow.q0e());
      } else {
        std::printf("error unknown mode %s\n", mode.c_str());
      }
    } catch (const std::exception &ex) {
      std::printf("throw %s\n", ex.what());
    }
    std::fflush(stdout);
  }
  return 0;
}
