"""CPU: the host side of the drop-in headers a generated flow pulls in through its def.hh --
RationalExpRegulator, the thermodynamic helpers, JSONValue, the math and utility helpers.

* RationalExpRegulator::get_f / get_df (built from the regulator's defining construction) equal
  the reference's per-order expressions, evaluated by tests/golden/make_regulator_golden.py from
  DiFfRG/include/DiFfRG/physics/regulators.hh, for orders 1..16 and three option sets, to 1e-13;
  RBdot and dq2RB equal forward-mode derivatives of RB.
* CothFiniteT / TanhFiniteT / SechFiniteT / CschFiniteT against the hyperbolic functions, their
  T/x -> 0 limits and overflow cases; dcothS, ddcothS, dddcothS, dtanhS, ddtanhS, dnB, ddnB, dnF
  against forward-mode derivatives of the function one order lower.
* JSONValue: nested paths, types, defaults, setters, errors, print/parse round trip, files.
* math and utilities: S_d, V_d, S_d_prec, is_close, sign, heaviside_theta, time_format, ...
The program is host code compiled by nvcc; it runs without a GPU.
"""
import json
import os
import subprocess

from diffrg_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))
COMPAT = os.path.join(B.INCLUDE, "gbint", "compat")

PROGRAM = r'''
#include <cmath>
#include <cstdio>
#include <fstream>
#include <string>
#include <DiFfRG/common/utils.hh>
#include <DiFfRG/physics/regulators.hh>
#include <DiFfRG/physics/thermodynamics.hh>
using namespace DiFfRG;
static int bad = 0;
static void check(bool ok, const char *what, double a = 0, double b = 0)
{
  if (!ok) {
    ++bad;
    std::printf("FAIL %s %.17g %.17g\n", what, a, b);
  }
}
static bool rel(double a, double b, double tol) { return std::fabs(a - b) <= tol * std::fmax(std::fabs(b), 1e-300); }
template <int N, int OPT> struct Opts;
#define OPTSET(I, C, B0) \
  template <int N> struct Opts<N, I> { static constexpr int order = N; constexpr static double c = C; constexpr static double b0 = B0; };
OPTSET(0, 2.0, 0.0)
OPTSET(1, 1.5, 0.25)
OPTSET(2, 3.0, 0.1)
template <int N, int O> void rational(double x, double f, double df)
{
  using R = RationalExpRegulator<Opts<N, O>>;
  check(rel(R::get_f(x), f, 1e-13), "get_f", R::get_f(x), f);
  check(rel(R::get_df(x), df, 1e-13), "get_df", R::get_df(x), df);
  // RBdot = d RB / d ln k at fixed q^2 (d k^2 = 2 k^2 d ln k); dq2RB = d RB / d q^2
  const double k2 = 1.3, q2 = x * k2;
  const autodiff::real rk = R::RB(autodiff::real(k2, 2 * k2), q2);
  check(rel(R::RBdot(k2, q2), autodiff::derivative(rk), 1e-11), "RBdot", R::RBdot(k2, q2), autodiff::derivative(rk));
  const autodiff::real rq = R::RB(k2, autodiff::real(q2, 1.0));
  check(rel(R::dq2RB(k2, q2), autodiff::derivative(rq), 1e-12), "dq2RB", R::dq2RB(k2, q2), autodiff::derivative(rq));
  check(rel(R::RF(k2, q2), std::sqrt(R::RB(k2, q2) + q2) - std::sqrt(q2), 1e-14), "RF");
}
template <int N, int O> void dispatch2(int n, int o, double x, double f, double df)
{
  if (n == N && o == O) rational<N, O>(x, f, df);
  if constexpr (O < 2) dispatch2<N, O + 1>(n, o, x, f, df);
}
template <int N> void dispatch(int n, int o, double x, double f, double df)
{
  dispatch2<N, 0>(n, o, x, f, df);
  if constexpr (N < 16) dispatch<N + 1>(n, o, x, f, df);
}
int main(int argc, char **argv)
{
  // golden RationalExpRegulator values on stdin: order option x f df
  int n, o;
  double x, f, df;
  int cases = 0;
  while (std::scanf("%d %d %lf %lf %lf", &n, &o, &x, &f, &df) == 5) {
    dispatch<1>(n, o, x, f, df);
    ++cases;
  }
  check(cases == 336, "golden cases read", cases, 336);

  // thermodynamics
  for (double T : {0.05, 0.3, 2.0})
    for (double e : {-3.0, -0.2, 0.01, 0.7, 5.0}) {
      check(rel(CothFiniteT(e, T), 1.0 / std::tanh(e / (2 * T)), 1e-15), "CothFiniteT");
      check(rel(TanhFiniteT(e, T), std::tanh(e / (2 * T)), 1e-15), "TanhFiniteT");
      check(rel(SechFiniteT(e, T), 1.0 / std::cosh(e / (2 * T)), 1e-15), "SechFiniteT");
      check(rel(CschFiniteT(e, T), 1.0 / std::sinh(e / (2 * T)), 1e-15), "CschFiniteT");
      check(rel(cothS(e, T), 1.0 + 2.0 * nB(e, T), 1e-12), "coth = 1 + 2 nB", cothS(e, T), 1.0 + 2.0 * nB(e, T));
      check(rel(tanhS(e, T), 1.0 - 2.0 * nF(e, T), 1e-12), "tanh = 1 - 2 nF");
      const autodiff::real E(e, 1.0);
      check(rel(dcothS(e, T), autodiff::derivative(cothS(E, T)), 1e-12), "dcothS", dcothS(e, T), autodiff::derivative(cothS(E, T)));
      check(rel(ddcothS(e, T), autodiff::derivative(dcothS(E, T)), 1e-12), "ddcothS");
      check(rel(dddcothS(e, T), autodiff::derivative(ddcothS(E, T)), 1e-11), "dddcothS");
      check(rel(dtanhS(e, T), autodiff::derivative(tanhS(E, T)), 1e-12), "dtanhS", dtanhS(e, T), autodiff::derivative(tanhS(E, T)));
      check(rel(ddtanhS(e, T), autodiff::derivative(dtanhS(E, T)), 1e-12), "ddtanhS");
      check(rel(dnB(e, T), autodiff::derivative(nB(E, T)), 1e-12), "dnB");
      check(rel(ddnB(e, T), autodiff::derivative(dnB(E, T)), 1e-11), "ddnB");
      check(rel(dnF(e, T), autodiff::derivative(nF(E, T)), 1e-12), "dnF");
      check(rel(autodiff::val(CothFiniteT(E, T)), CothFiniteT(e, T), 1e-15), "CothFiniteT(dual) value");
    }
  check(CothFiniteT(0.4, 0.0) == 1.0 && CothFiniteT(-0.4, 0.0) == -1.0, "CothFiniteT T = 0");
  check(TanhFiniteT(2.0, 1e-18) == 1.0 && TanhFiniteT(-2.0, 0.0) == -1.0, "TanhFiniteT T/x -> 0");
  check(SechFiniteT(2000.0, 0.1) == 0.0 && CschFiniteT(2000.0, 0.1) == 0.0, "Sech/Csch overflow -> 0");
  const cuda::std::complex<double> z(0.8, 0.3);
  check(std::abs(cuda::std::abs(CothFiniteT(z, 0.2) - 1.0 / cuda::std::tanh(z / 0.4))) < 1e-14, "CothFiniteT complex");

  // JSONValue
  const std::string path = argc > 1 ? argv[1] : "settings.json";
  JSONValue j(std::string(R"({"a": {"b": 2.5, "n": 7, "s": "txt", "t": true, "arr": [1, 2, {"z": -3}]},
                              "esc": "q\"\\é"})"));
  check(j.get_double("/a/b") == 2.5 && j.get_uint("/a/n") == 7u && j.get_int("a/n") == 7, "json numbers");
  check(j.get_string("/a/s") == "txt" && j.get_bool("/a/t"), "json string/bool");
  check(j.get_int("/a/arr/2/z") == -3, "json array path");
  check(j.get_double("/a/missing", 4.0) == 4.0 && j.get_uint("/x/y", 3u) == 3u, "json defaults");
  check(j.get_string("/esc") == "q\"\\\xc3\xa9", "json escapes");
  bool threw = false;
  try {
    j.get_double("/a/missing");
  } catch (const std::runtime_error &) {
    threw = true;
  }
  check(threw, "json missing key throws");
  j.set_double("/new/deep/v", 0.125);
  j.set_uint("/a/n", 9u);
  j.set_string("/a/s", "other");
  check(j.get_double("/new/deep/v") == 0.125 && j.get_uint("/a/n") == 9u && j.get_string("/a/s") == "other", "json setters");
  {
    std::ofstream fo(path);
    j.print(fo);
  }
  JSONValue back(path);
  check(back == j && back.get_double("/new/deep/v") == 0.125, "json file round trip");
  JSONValue copy = j;
  copy.set_int("/a/n", 1);
  check(j.get_uint("/a/n") == 9u, "json copies are deep");

  // math and utilities
  const double pi = 3.14159265358979323846;
  check(rel(S_d(4), 2 * pi * pi, 1e-15) && rel(S_d(3), 4 * pi, 1e-15) && rel(S_d_prec<double>(5), 8 * pi * pi / 3, 1e-15), "S_d");
  check(rel(V_d(3), 4 * pi / 3, 1e-15) && rel(V_d(2, 2.0), 4 * pi, 1e-15), "V_d");
  check(is_close(1.0, 1.0 + 1e-16) && !is_close(1.0, 1.0 + 1e-10) && is_close(1.0, 1.001, 1e-2), "is_close");
  check(sign(-2.0) == -1.0 && sign(0.0) == 1.0 && heaviside_theta(-1e-300) == 0.0 && heaviside_theta(0.0) == 1.0, "sign/theta");
  check(time_format(59) == "59s" && time_format(125) == "2min5s" && time_format(3723) == "1h2min3s", "time_format");
  check(time_format_ms(999) == "999ms" && time_format_ms(1250) == "1s250ms" && time_format_ms(3723000) == "1h2min", "time_format_ms");
  check(strip_name("a b-c.(d)") == "abcd" && has_suffix("flow.json", ".json") && make_folder("out") == "out/", "strings");
  const auto arr = string_to_double_array("1,2.5,-3");
  check(arr.size() == 3 && arr[1] == 2.5 && arr[2] == -3.0, "string_to_double_array");
  check(getWithPrecision(2, 3.14159) == "3.14", "getWithPrecision");
  int seen = 0;
  constexpr_for<0, 4, 1>([&](auto i) { seen += (int)i; });
  check(seen == 6, "constexpr_for");

  std::printf("BAD %d\n", bad);
  return bad ? 1 : 0;
}
'''


def test_boundary_headers_host(tmp_path):
    src = tmp_path / "boundary.cu"
    src.write_text(PROGRAM)
    exe = str(tmp_path / "boundary")
    cmd = [B.nvcc(), "-std=c++20", "-O1", "--expt-relaxed-constexpr", "-I", COMPAT, "-I", B.INCLUDE] + B.ARCH + \
        [str(src), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-5000:]
    gold = json.load(open(os.path.join(HERE, "golden", "rational_exp_regulator.json")))
    optidx = {(2.0, 0.0): 0, (1.5, 0.25): 1, (3.0, 0.1): 2}
    lines = ["%d %d %r %r %r" % (c["order"], optidx[(c["c"], c["b0"])], c["x"], c["f"], c["df"]) for c in gold["cases"]]
    r = subprocess.run([exe, str(tmp_path / "settings.json")], input="\n".join(lines) + "\n", capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert r.stdout.strip().endswith("BAD 0")
