"""CPU: the C++ drop-in headers (integrators, interpolators, autodiff, regulators, fan-out
helpers, kernel math, the forwarding headers at the reference's include paths) compile for
sm_103a in a user translation unit -- the GPU test driver tests/cpp/test_integrators.cu, and a
small unit that includes every forwarding header by its reference path.  nvcc cross-compiles
without a GPU; nothing runs."""
import os
import subprocess

from diffrg_gb300 import build as B
from diffrg_gb300 import cppapi


def test_gpu_test_driver_compiles():
    out = cppapi.build_tests()
    assert os.path.exists(out)


def test_every_forwarding_header_compiles(tmp_path):
    compat = os.path.join(B.INCLUDE, "gbint", "compat")
    heads = sorted(os.path.relpath(os.path.join(d, f), compat) for d, _, fs in os.walk(compat) for f in fs
                   if f.endswith(".hh"))
    assert len(heads) >= 45
    src = tmp_path / "all_headers.cu"
    src.write_text("".join('#include <%s>\n' % h for h in heads) + '#include "gbint/kernel_math.hh"\n'
                   "int main() { return DiFfRG::powr<2>(1.0) == 1.0 ? 0 : 1; }\n")
    cmd = [B.nvcc(), "-std=c++17", "--expt-relaxed-constexpr", "-I", compat, "-I", B.INCLUDE] + B.ARCH + \
        ["-c", str(src), "-o", str(tmp_path / "all_headers.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def test_flow_equations_with_dual_results(tmp_path):
    """FlowEquations over gbint::dual results (gbint/autodiff.hh next to gbint/flow_equations.hh,
    host code of an nvcc unit): the jacobian rules are taken and the derivative is the loop
    integral of the derivative of the integrand.  Host code only; runs without a GPU."""
    src = tmp_path / "flow_dual.cu"
    src.write_text(r'''
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include "gbint/autodiff.hh"
#include <DiFfRG/physics/flow_equations.hh>
struct Json {
  std::map<std::string, double> v;
  unsigned get_uint(const std::string &p) const { return (unsigned)v.at(p); }
  double get_double(const std::string &p) const { return v.at(p); }
  int get_int(const std::string &p) const { return (int)v.at(p); }
};
struct Flow : DiFfRG::FlowEquations {
  Flow(const Json &j) : FlowEquations(j, [](double q2) { return std::exp(-q2); }) {}
  double xe() const { return x_extent; }
  unsigned jo() const { return jac_x_quadrature_order; }
};
int main() {
  Json j;
  j.v = {{"/integration/x_quadrature_order", 16}, {"/integration/angle_quadrature_order", 8},
         {"/integration/jacobian_quadrature_factor", 1.5}, {"/integration/x_extent_tolerance", 1e-3},
         {"/output/verbosity", 0}};
  Flow flow(j);
  flow.set_k(0.9);
  const double a = 0.7;
  const autodiff::real A = gbint::seed(a);
  const autodiff::real r = flow.integrate<autodiff::real, 4>([&](double q2) { return gbint::exp(-A * q2); });
  const DiFfRG::QGauss<1> jq(flow.jo());
  const double v = DiFfRG::LoopIntegrals::integrate<double, 4>([&](double q2) { return std::exp(-a * q2); }, jq,
                                                               flow.xe(), 0.9);
  const double dv = DiFfRG::LoopIntegrals::integrate<double, 4>(
      [&](double q2) { return -q2 * std::exp(-a * q2); }, jq, flow.xe(), 0.9);
  const bool ok = flow.jo() == 24 && std::fabs(gbint::val(r) - v) <= 1e-15 * std::fabs(v) &&
                  std::fabs(gbint::derivative(r) - dv) <= 1e-14 * std::fabs(dv);
  std::printf("%d %.17g %.17g %.17g %.17g\n", (int)ok, gbint::val(r), v, gbint::derivative(r), dv);
  return ok ? 0 : 1;
}
''')
    compat = os.path.join(B.INCLUDE, "gbint", "compat")
    exe = str(tmp_path / "flow_dual")
    cmd = [B.nvcc(), "-std=c++17", "--expt-relaxed-constexpr", "-I", compat, "-I", B.INCLUDE] + B.ARCH + \
        [str(src), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
