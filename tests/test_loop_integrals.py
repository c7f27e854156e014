"""Host loop integrals and flow-equation extent fits (include/gbint/loop_integrals.hh,
include/gbint/flow_equations.hh) -- CPU tests, no GPU.

The C++ driver tests/cpp/test_loop_integrals.cc is compiled with g++ alone.  Checks:
  * QGauss<1> against the reference's constexpr Gauss-Legendre tables (tests/golden/gl_tables.json);
  * every LoopIntegrals function against the closed forms of the reference's own tests
    (DiFfRG/tests/physics/test_loop_integrals.cc:16-289, same integrands, rules, parameter ranges
    and tolerances; seeded draws stand in for Catch2's GENERATE(random(...)));
  * every LoopIntegrals function, double and std::complex results, against the oracle's numpy
    restatement (oracle/loop_integrals.py) at 1e-12 relative;
  * results independent of the thread count (byte-identical output with 1 and 8 threads);
  * FlowEquations / FlowEquationsFiniteT extent fits equal to the restated fit
    (flow_equations.cc:54-285): the same number of 1.15 steps, hence the same doubles; the
    all-zero probe; the error for a diverging integrand; the jacobian rules for marked types.
"""
from __future__ import annotations

import json
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import loop_integrals as L

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cpp", "test_loop_integrals.cc")
PI = math.pi


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("loop") / "test_loop_integrals")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-pthread", "-Wall", "-Wextra", "-Werror", "-I",
                        os.path.join(ROOT, "include"), SRC, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


def run(exe, lines, threads=None):
    env = dict(os.environ)
    if threads is not None:
        env["GBINT_HOST_THREADS"] = str(threads)
    r = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    out = r.stdout.strip().split("\n")
    assert len(out) == len(lines), r.stdout
    return out


def li_line(fn, *, nt=0, d=4, nx=64, ncos=0, nm=0, x_extent=1.0, k=1.0, m_extent=1.0, m_order=0, T=0.0, zeta=0.0,
            a=(1,), c=(1,), b=(1,), e=(1,)):
    pad = lambda v, n: list(v) + [0.0] * (n - len(v))
    vals = [nt, d, nx, ncos, nm, repr(x_extent), repr(k), repr(m_extent), m_order, repr(T), repr(zeta)]
    vals += [repr(float(v)) for v in pad(a, 8) + pad(c, 4) + pad(b, 4) + pad(e, 4)]
    return "li %s %s" % (fn, " ".join(str(v) for v in vals))


def parse_c(s):
    re_, im = s.split()
    return complex(float(re_), float(im))


def S(d):
    return 2.0 * PI ** (d / 2.0) / math.gamma(d / 2.0)


def radial_closed(a, d, q_extent):
    """int_0^q_extent P(q^2) q^(d-1) dq for P = sum a_i t^i."""
    return sum(ai * q_extent ** (2 * i + d) / (2 * i + d) for i, ai in enumerate(a))


def poly_int(c, lo, hi):
    return sum(ci * (hi ** (i + 1) - lo ** (i + 1)) / (i + 1) for i, ci in enumerate(c))


def pv(c):
    return lambda t: sum(ci * t ** i for i, ci in enumerate(c))


# ---------------------------------------------------------------------------------------------


def test_qgauss_matches_reference_gl_tables(driver):
    gold = json.load(open(os.path.join(HERE, "golden", "gl_tables.json")))["tables"]
    orders = sorted(int(n) for n in gold)
    out = run(driver, ["gl %d" % n for n in orders])
    for n, line in zip(orders, out):
        v = np.array([float(t) for t in line.split()])
        x, w = v[:n], v[n:]
        np.testing.assert_allclose(x, [float(s) for s in gold[str(n)]["x"]], rtol=0, atol=4e-16)
        np.testing.assert_allclose(w, [float(s) for s in gold[str(n)]["w"]], rtol=0, atol=4e-16)


def _rng_cases(seed, n):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        yield rng


def test_closed_forms_of_the_reference_tests(driver):
    """The six quadrature test cases of DiFfRG/tests/physics/test_loop_integrals.cc:16-289."""
    lines, expect, tols = [], [], []
    for rng in _rng_cases(20240601, 6):
        for dim in (1, 2, 3, 4):
            a = list(rng.uniform(-1, 1, 8))
            if dim == 1:
                a[0] = 0.0
            k = rng.uniform(0, 1)
            xe = rng.uniform(1, 2)
            qe = math.sqrt(xe * k * k)
            ref = S(dim) * radial_closed(a, dim, qe) / (2 * PI) ** dim
            lines.append(li_line("integrate", d=dim, nx=64, x_extent=xe, k=k, a=a))
            expect.append(ref)
            tols.append(1e-6)
            if dim >= 2:
                c = list(rng.uniform(-1, 1, 4))
                ref = S(dim) / 2 * radial_closed(a, dim, qe) / (2 * PI) ** dim * poly_int(c, -1, 1)
                lines.append(li_line("angle", d=dim, nx=64, ncos=5, x_extent=xe, k=k, a=a, c=c))
                expect.append(ref)
                tols.append(1e-6)
                # q0 integral (spatial dimension ds = dim - 1)
                ds = dim - 1
                a2 = list(a)
                if dim == 2:
                    a2[0] = 0.0
                b = list(rng.uniform(-1, 1, 4))
                q0e = rng.uniform(1e-2, 1)
                rad = S(ds) * radial_closed(a2, ds, qe) / (2 * PI) ** ds
                lines.append(li_line("sii", d=dim, nx=64, nm=7, x_extent=xe, k=k, m_extent=q0e, a=a2, b=b))
                expect.append(rad * poly_int(b, -q0e, q0e) / (2 * PI))
                tols.append(1e-6)
                lines.append(li_line("saii", d=dim, nx=64, ncos=5, nm=7, x_extent=xe, k=k, m_extent=q0e, a=a2,
                                     c=c, b=b))
                expect.append(rad / 2 * poly_int(c, -1, 1) * poly_int(b, -q0e, q0e) / (2 * PI))
                tols.append(1e-6)
                # Matsubara sums: sum_n T |n|^-zeta (n != 0) + T = T (1 + 2 zeta(z))
                from scipy.special import zeta as rzeta
                m_order = int(rng.integers(30, 51))
                q0e = 2 * PI * (m_order + rng.uniform(500, 700))
                z = rng.uniform(3, 6)
                T = rng.uniform(1e-2, 1)
                lines.append(li_line("sis", d=dim, nx=64, nm=32, x_extent=xe, k=k, m_extent=q0e, m_order=m_order,
                                     T=T, zeta=z, a=a2))
                expect.append(rad * (1 + 2 * rzeta(z)) * T)
                tols.append(1e-5)
                lines.append(li_line("sais", d=dim, nx=64, ncos=5, nm=32, x_extent=xe, k=k, m_extent=q0e,
                                     m_order=m_order, T=T, zeta=z, a=a2, c=c))
                expect.append(rad / 2 * poly_int(c, -1, 1) * (1 + 2 * rzeta(z)) * T)
                tols.append(1e-5)
    out = run(driver, lines)
    for line, got, ref, tol in zip(lines, out, expect, tols):
        v = parse_c(got).real
        # DiFfRG's is_close(reference, integral, tol): absolute or relative
        assert abs(v - ref) <= tol or abs(v - ref) <= tol * max(abs(v), abs(ref)), (line, v, ref)


def test_two_angle_closed_form(driver):
    """two_angle_integrate computes the integral its documentation states (phi weights of the phi
    rule): exact for polynomial integrands in even d, where the x integrand P(x) x^((d-2)/2) is a
    polynomial too."""
    rng = np.random.default_rng(7)
    lines, expect = [], []
    for d in (4, 6):
        a = list(rng.uniform(-1, 1, 6))
        c = list(rng.uniform(-1, 1, 4))
        e = list(rng.uniform(-1, 1, 4))
        k, xe = 0.8, 1.7
        qe = math.sqrt(xe) * k
        rad = S(d) * radial_closed(a, d, qe) / (2 * PI) ** d
        lines.append(li_line("two_angle", d=d, nx=64, ncos=6, x_extent=xe, k=k, a=a, c=c, e=e))
        expect.append(rad * 0.5 * poly_int(c, -1, 1) * poly_int(e, 0, 2 * PI) / (2 * PI))
    out = run(driver, lines)
    for line, got, ref in zip(lines, out, expect):
        assert abs(parse_c(got).real - ref) <= 1e-12 * abs(ref), (line, got, ref)


ORACLE = {
    "integrate": lambda f, p: L.integrate(lambda q2: f["a"](q2), p["d"], p["nx"], p["x_extent"], p["k"]),
    "angle": lambda f, p: L.angle_integrate(lambda q2, c: f["a"](q2) * f["c"](c), p["d"], p["nx"], p["x_extent"],
                                            p["k"], p["ncos"]),
    "two_angle": lambda f, p: L.two_angle_integrate(lambda q2, c, ph: f["a"](q2) * f["c"](c) * f["e"](ph), p["d"],
                                                    p["nx"], p["x_extent"], p["k"], p["ncos"]),
    "three_angle": lambda f, p: L.three_angle_integrate(
        lambda q2, c1, c2, ph: f["a"](q2) * f["c"](c1) * f["b"](c2) * f["e"](ph), p["d"], p["nx"], p["x_extent"],
        p["k"], p["ncos"]),
    "sii": lambda f, p: L.spatial_integrate_and_integrate(lambda q2, q0: f["a"](q2) * f["q"](q0), p["d"], p["nx"],
                                                          p["x_extent"], p["k"], p["nm"], p["m_extent"]),
    "saii": lambda f, p: L.spatial_angle_integrate_and_integrate(
        lambda q2, c, q0: f["a"](q2) * f["c"](c) * f["q"](q0), p["d"], p["nx"], p["x_extent"], p["k"], p["ncos"],
        p["nm"], p["m_extent"]),
    "sis": lambda f, p: L.spatial_integrate_and_sum(lambda q2, q0: f["a"](q2) * f["q"](q0), p["d"], p["nx"],
                                                    p["x_extent"], p["k"], p["m_order"], p["nm"], p["m_extent"],
                                                    p["T"]),
    "sais": lambda f, p: L.spatial_angle_integrate_and_sum(
        lambda q2, c, q0: f["a"](q2) * f["c"](c) * f["q"](q0), p["d"], p["nx"], p["x_extent"], p["k"], p["ncos"],
        p["m_order"], p["nm"], p["m_extent"], p["T"]),
    "sum": lambda f, p: L.loop_sum(lambda q0: f["q"](q0), p["m_order"], p["nm"], p["m_extent"], p["T"]),
}

MIN_D = {"integrate": 1, "angle": 2, "two_angle": 3, "three_angle": 4, "sii": 2, "saii": 2, "sis": 2, "sais": 2,
         "sum": 4}


def _oracle_cases(seed):
    rng = np.random.default_rng(seed)
    cases = []
    for fn in ORACLE:
        for d in (1, 2, 3, 4, 5):
            if d < MIN_D[fn] or (fn == "sum" and d != 4):
                continue
            for nt in (0, 1):
                p = dict(d=d, nt=nt, nx=int(rng.integers(8, 40)), ncos=int(rng.integers(3, 9)),
                         nm=int(rng.integers(4, 20)), x_extent=float(rng.uniform(0.5, 3)), k=float(rng.uniform(0.2, 2)),
                         m_extent=float(rng.uniform(0.5, 40)), m_order=int(rng.integers(0, 12)),
                         T=float(rng.choice([0.0, rng.uniform(0.05, 1.0)])), zeta=0.0)
                if fn in ("sis", "sais", "sum") and p["T"] > 0:
                    p["m_extent"] = 2 * PI * p["T"] * (p["m_order"] + 1) + float(rng.uniform(1, 30))
                coef = {kk: list(rng.uniform(-1, 1, n)) for kk, n in (("a", 6), ("c", 4), ("b", 4), ("e", 4))}
                if d <= 2:
                    coef["a"][0] = 0.0  # x^((d-2)/2) at x -> 0
                cases.append((fn, p, coef))
    return cases


def _funcs(coef):
    f = {kk: pv(v) for kk, v in coef.items()}
    f["q"] = f["b"]
    return f


@pytest.mark.parametrize("seed", [11, 12])
def test_every_loop_integral_matches_the_oracle(driver, seed):
    cases = _oracle_cases(seed)
    lines = [li_line(fn, nt=p["nt"], d=p["d"], nx=p["nx"], ncos=p["ncos"], nm=p["nm"], x_extent=p["x_extent"], k=p["k"],
                     m_extent=p["m_extent"], m_order=p["m_order"], T=p["T"], a=c["a"], c=c["c"], b=c["b"], e=c["e"])
             for fn, p, c in cases]
    out = run(driver, lines)
    for (fn, p, c), got in zip(cases, out):
        ref = complex(ORACLE[fn](_funcs(c), p))
        if p["nt"]:
            ref = ref * (1 + 0.5j)
        v = parse_c(got)
        scale = max(abs(ref), 1e-300)
        assert abs(v - ref) <= 1e-12 * scale, (fn, p, v, ref)


def test_two_angle_differs_from_the_reference_weighting(driver):
    """The reference's phi weight (the cos node's weight) gives another number; ours is the
    documented integral.  Both are restated by the oracle."""
    p = dict(d=4, nx=16, ncos=5, x_extent=1.3, k=0.9)
    f = lambda q2, c, ph: (1 + q2) * (0.5 + c * c) * (1 + 0.1 * ph)
    ours = L.two_angle_integrate(f, p["d"], p["nx"], p["x_extent"], p["k"], p["ncos"])
    theirs = L.two_angle_integrate(f, p["d"], p["nx"], p["x_extent"], p["k"], p["ncos"], reference_phi_weight=True)
    got = parse_c(run(driver, [li_line("two_angle", d=4, nx=16, ncos=5, x_extent=1.3, k=0.9, a=(1, 1), c=(0.5, 0, 1),
                                       e=(1, 0.1))])[0]).real
    assert abs(got - ours) <= 1e-13 * abs(ours)
    assert abs(ours - theirs) > 1e-3 * abs(ours)


def test_results_do_not_depend_on_the_thread_count(driver):
    lines = [
        li_line("angle", d=4, nx=256, ncos=64, x_extent=2.0, k=0.7, a=(0.3, -0.2, 0.1), c=(1, 0.5)),
        li_line("sais", nt=1, d=4, nx=64, ncos=5, nm=32, x_extent=1.5, k=0.8, m_extent=300.0, m_order=40, T=0.3,
                zeta=4.5, a=(0.1, 0.4), c=(1, -0.3)),
        li_line("three_angle", d=4, nx=40, ncos=12, x_extent=1.2, k=1.1, a=(1, 0.2), c=(1, 0.1), b=(1, 0.3),
                e=(1, 0.05)),
        li_line("sii", d=3, nx=512, nm=64, x_extent=1.1, k=1.0, m_extent=5.0, a=(0.0, 1.0), b=(1, 0, 0.2)),
    ]
    one = run(driver, lines, threads=1)
    many = run(driver, lines, threads=8)
    assert one == many


def test_sum_variants_at_zero_temperature_are_the_integrals(driver):
    common = dict(d=4, nx=24, ncos=5, nm=12, x_extent=1.4, k=0.6, m_extent=3.0, m_order=7, a=(1, 0.5), c=(1, 0.2),
                  b=(1, 0, -0.1))
    out = run(driver, [li_line("sis", T=0.0, **common), li_line("sii", **common), li_line("sais", T=0.0, **common),
                       li_line("saii", **common)])
    assert out[0] == out[1] and out[2] == out[3]


# ---------------------------------------------------------------------------------------------
# FlowEquations extent fits

FX = {"gauss": lambda q2: np.exp(-q2), "rational": lambda q2: 1.0 / (1.0 + q2) ** 4,
      "zero": lambda q2: np.where(q2 < 1.0, 1.0 - q2, 0.0), "gauss0": lambda q0: np.exp(-q0 * q0),
      "rational0": lambda q0: 1.0 / (1.0 + q0 * q0) ** 4}


@pytest.mark.parametrize("order,tol,fx", [(32, 1e-3, "gauss"), (16, 1e-4, "rational"), (24, 1e-6, "gauss"),
                                          (32, 1e-3, "zero")])
def test_x_extent_fit_matches_the_restated_fit(driver, order, tol, fx):
    got = float(run(driver, ["fe %d 8 2 %r %s" % (order, tol, fx)])[0])
    ref, _ = L.fit_x_extent(FX[fx], order, tol)
    assert got == ref
    if fx == "zero":
        assert got == 1.0


def test_x_extent_fit_reports_a_diverging_integrand(driver):
    out = run(driver, ["fe 16 8 2 1e-3 grow"])[0]
    assert out.startswith("throw Cannot reach requested precision for x_extent"), out
    with pytest.raises(L.ExtentError):
        L.fit_x_extent(lambda q2: np.exp(q2), 16, 1e-3)


@pytest.mark.parametrize("x0s,q0s", [(8, 8), (0, 4), (3, 0)])
def test_finite_T_extent_fits_match_the_restated_fits(driver, x0s, q0s):
    line = "fet 32 8 2 1e-3 16 1e-4 %d 16 1e-3 %d 0.1 gauss rational0 gauss0" % (x0s, q0s)
    xe, x0e, q0e = (float(t) for t in run(driver, [line])[0].split())
    rxe, _ = L.fit_x_extent(FX["gauss"], 32, 1e-3)
    assert xe == rxe
    assert x0e == (L.fit_x0_extent(FX["rational0"], 16, 1e-4, rxe)[0] if x0s else 0.0)
    assert q0e == (L.fit_q0_extent(FX["gauss0"], 16, 1e-3, rxe)[0] if q0s else 0.0)


def test_print_parameters_layout(driver):
    """The parameter logs in the reference's layout (S/physics/flow_equations.cc print_parameters):
    FlowEquations labels right-aligned in 40 columns and values in 10; FlowEquationsFiniteT labels
    right-aligned in 10 columns, values as printed."""
    line = run(driver, ["fe 16 8 2 1e-3 gauss print"])[0]
    xe = float(run(driver, ["fe 16 8 2 1e-3 gauss"])[0])
    rows = [("x_quadrature_order", "16"), ("jac_x_quadrature_order", "32"), ("x_extent", "%g" % xe),
            ("angle_quadrature_order", "8"), ("jac_angle_quadrature_order", "16")]
    want = "[log] FlowEquations:" + "".join("|%40s%10s" % (k + ": ", v) for k, v in rows) + "|"
    assert line == want, (line, want)
    line = run(driver, ["fet 32 8 2 1e-3 16 1e-4 0 16 1e-3 0 0.1 gauss rational0 gauss0 print"])[0]
    assert line.startswith("[log] FlowEquationsFiniteT:|x_quadrature_order: 32|jac_x_quadrature_order: 64|")
    assert line.endswith("|jac_angle_quadrature_order: 16|%10s0.1|" % "T: "), line


def test_marked_result_types_take_the_jacobian_rules(driver):
    a, b = (float(t) for t in run(driver, ["jac 16 8 2 1e-3 rational 0.8"])[0].split())
    assert a == b


def test_dealii_rule_is_taken_when_dealii_is_included_first(tmp_path):
    """With deal.II's quadrature_lib.h included first, DiFfRG::QGauss is deal.II's rule: a
    stand-in with deal.II's interface (Point<1> points, include guard dealii_quadrature_lib_h)
    goes through LoopIntegrals and FlowEquations unchanged."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "dealii_rule.cc"
    src.write_text(r'''
#include <cmath>
#include <cstdio>
#include <map>
#include <string>
#include <vector>
#include "gbint/gl_rule.hh"
#define dealii_quadrature_lib_h
namespace dealii {
  template <int dim> struct Point { double c[dim]; double operator[](unsigned i) const { return c[i]; } };
  template <int dim> class QGauss {
  public:
    explicit QGauss(unsigned n) : tag(7) {
      std::vector<double> x; gbint::gl_rule01((int)n, x, w);
      for (double v : x) p.push_back(Point<1>{{v}});
    }
    const std::vector<Point<1>> &get_points() const { return p; }
    const std::vector<double> &get_weights() const { return w; }
    unsigned size() const { return (unsigned)w.size(); }
    int tag;
  private:
    std::vector<Point<1>> p; std::vector<double> w;
  };
}
#include <DiFfRG/physics/flow_equations.hh>
struct Json {
  std::map<std::string, double> v;
  unsigned get_uint(const std::string &k) const { return (unsigned)v.at(k); }
  double get_double(const std::string &k) const { return v.at(k); }
  int get_int(const std::string &k) const { return (int)v.at(k); }
};
struct Flow : DiFfRG::FlowEquations {
  Flow(const Json &j) : FlowEquations(j, [](double q2) { return std::exp(-q2); }) {}
  int tag() const { return x_quadrature.tag; }
};
int main() {
  static_assert(std::is_same_v<DiFfRG::QGauss<1>, dealii::QGauss<1>>, "deal.II's rule");
  Json j;
  j.v = {{"/integration/x_quadrature_order", 16}, {"/integration/angle_quadrature_order", 8},
         {"/integration/jacobian_quadrature_factor", 2}, {"/integration/x_extent_tolerance", 1e-3},
         {"/output/verbosity", 0}};
  Flow f(j);
  const double v = f.angle_integrate<double, 4>([](double q2, double c) { return (1 + q2) * (1 + c * c); });
  std::printf("%d %.17g\n", f.tag(), v);
  return f.tag() == 7 && std::isfinite(v) ? 0 : 1;
}
''')
    exe = str(tmp_path / "dealii_rule")
    r = subprocess.run([gxx, "-std=c++17", "-O1", "-pthread", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "include", "gbint", "compat"), str(src), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr


def test_reference_phi_weighting_on_request(tmp_path):
    """-DGBINT_LOOP_REFERENCE_PHI_WEIGHT gives the reference's two_angle_integrate
    (loop_integrals.hh:180-181), as the oracle restates it literally."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "ref_phi")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-pthread", "-DGBINT_LOOP_REFERENCE_PHI_WEIGHT", "-I",
                        os.path.join(ROOT, "include"), SRC, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    f = lambda q2, c, ph: (1 + q2) * (0.5 + c * c) * (1 + 0.1 * ph)
    theirs = L.two_angle_integrate(f, 4, 16, 1.3, 0.9, 5, reference_phi_weight=True)
    got = parse_c(run(exe, [li_line("two_angle", d=4, nx=16, ncos=5, x_extent=1.3, k=0.9, a=(1, 1), c=(0.5, 0, 1),
                                    e=(1, 0.1))])[0]).real
    assert abs(got - theirs) <= 1e-13 * abs(theirs)
