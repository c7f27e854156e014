"""The DiFfRG-compatible C++ class templates (include/gbint/integrators.hh) on the GPU.

A user translation unit (tests/cpp/test_integrators.cu) instantiates every integrator family
with a polynomial KERNEL, as the reference's integrator tests do, for NT = double and float.
Each value is checked against the FP64 oracle (same quadrature: 1e-12 for double, 2e-5 for
float; plain FP32 user kernels) and against the closed-form integral (the reference's tolerances).
"""
import math
import os
import subprocess

import numpy as np
import pytest

from kat import CASES, analytic, random_args

pytestmark = pytest.mark.gpu

FAM = {"1D": 1, "ANGLE": 2, "3D": 3, "4D2ANG": 4, "4D": 5, "CART1": 6, "CART2": 7, "CART3": 8, "2DPQ0": 9,
       "2DPX0": 10, "3DPQ0": 11, "3DPX0": 12, "FTQ0": 13, "ANGLE_FTQ0": 14, "4D_FTQ0": 15, "FTX0": 16,
       "ANGLE_FTX0": 17, "4D_FTX0": 18, "CONST": 19}


@pytest.fixture(scope="module")
def binary():
    from diffrg_gb300 import cppapi

    return cppapi.build_tests()


def make_case(fam, seed):
    rng = np.random.default_rng(seed)
    kw = dict(CASES[fam])
    n = kw.pop("n")
    d = kw.pop("d")
    k = rng.uniform(0.3, 1.0)
    xe = rng.uniform(1.0, 2.0)
    T = kw.get("T", 0.0)
    args = random_args(rng, q0_rational=(T, rng.uniform(0.8, 1.2))) if fam.endswith("FTQ0") else random_args(rng)
    if fam.endswith("FTX0"):
        kw["x0_extent"] = kw["x0_summands"] * 10 * 2 * math.pi * T / k * 1.5 + 1000.0 / k
    return n, d, k, xe, args, kw


def line(fam, n, d, k, xe, args, kw, prec):
    nn = list(n) + [0] * (4 - len(n))
    vals = [FAM[fam], d] + nn + [xe, kw.get("x0_extent", 0.0), kw.get("x0_summands", 0), kw.get("T", 0.0), k, prec]
    return " ".join(repr(float(v)) if isinstance(v, float) else str(int(v)) for v in vals) + " " + \
        " ".join(repr(float(a)) for a in args)


def run(binary, lines, extra=()):
    r = subprocess.run([binary] + list(extra), input="\n".join(lines) + "\n", capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.strip().splitlines()


def test_all_families_double_and_float(binary, oracle):
    from test_oracle_families import oracle_family

    fams = list(CASES)
    cases = [make_case(f, 31 + i) for i, f in enumerate(fams)]
    lines = [line(f, *c, prec=p) for p in (0, 1) for f, c in zip(fams, cases)]
    out = run(binary, lines)
    vals = np.array([float(v) for v in out[:len(lines)]])
    nf = len(fams)
    for i, (f, (n, d, k, xe, args, kw)) in enumerate(zip(fams, cases)):
        ref = oracle_family(oracle, f, n, d, k, xe, args, kw)
        ana = analytic(f, args, k, d=d, x_extent=xe, **kw)
        got64, got32 = vals[i], vals[nf + i]
        assert abs(got64 - ref) <= 1e-12 * max(abs(ref), 1e-3), (f, got64, ref)
        assert abs(got32 - ref) <= 2e-5 * max(abs(ref), 1e-3), (f, got32, ref)
        tol = 5e-5 if f.endswith("FTQ0") else 1e-4
        assert abs(got64 - ana) <= tol * max(1.0, abs(ana)), (f, got64, ana)


def test_interpolators_inside_user_kernels(binary):
    """TexLinearInterpolator1D / LinearInterpolator1D objects passed into a KERNEL: device
    interpolation equals the interpolators' host branch summed over the same quadrature, and
    update() reaches the next launch."""
    out = run(binary, [], extra=["--interp"])
    rows = [l.split()[1:] for l in out if l.startswith("INTERP")]
    assert len(rows) == 4
    for a, b in rows:
        assert abs(float(a) - float(b)) <= 1e-6 * abs(float(b)), (a, b)
    assert abs(float(rows[3][0]) - float(rows[1][0])) > 1e-3 * abs(float(rows[1][0]))


def test_request_futures_match_get(binary):
    out = run(binary, [], extra=["--requests"])
    reqs = [l.split() for l in out if l.startswith("REQ")]
    assert len(reqs) == 32
    for _, a, b in reqs:
        assert float(a) == float(b)


def test_3d_and_stacked_interpolators(binary):
    """TexLinearInterpolator3D / LinearInterpolator3D on a CoordinatePackND of three axes and
    TexLinearInterpolator1DStack on BosonicCoordinates1DFiniteT: the device branch equals the
    host branch, and both reproduce data that are multilinear in the grid index exactly
    (FP32 storage of the Tex* data: 1e-6), including clamping and the folding of frequencies
    above the stored modes."""
    out = run(binary, [], extra=["--interp3"])
    rows = {k: [list(map(float, l.split()[1:])) for l in out if l.startswith(k + " ")]
            for k in ("LIN3", "TEX3", "CLAMP3", "STACK")}
    assert len(rows["LIN3"]) == 40 and len(rows["TEX3"]) == 40 and len(rows["STACK"]) == 24
    for dev, host, ana in rows["LIN3"]:
        assert abs(dev - host) <= 1e-14 * max(1, abs(ana)) and abs(dev - ana) <= 1e-12 * max(1, abs(ana))
    for dev, host, ana in rows["TEX3"]:
        assert abs(dev - host) <= 1e-6 * max(1, abs(ana)) and abs(dev - ana) <= 2e-6 * max(1, abs(ana))
    for dev, ana in rows["CLAMP3"]:
        assert abs(dev - ana) <= 1e-12 * max(1, abs(ana))
    for dev, host, ana in rows["STACK"]:
        assert abs(dev - host) <= 1e-6 * abs(ana) and abs(dev - ana) <= 2e-6 * abs(ana)


def test_complex_result_type(binary):
    """NT = cuda::std::complex<double/float>: the components are reduced separately and equal
    the two real integrals (FP64 to rounding, FP32 to 1e-5)."""
    out = run(binary, [], extra=["--complex"])
    rows = [list(map(float, l.split()[1:])) for l in out if l.startswith("CPLX")]
    assert len(rows) == 3
    for re, im, ra, rb, fre, fim in rows:
        assert abs(re - ra) <= 1e-13 * max(1, abs(ra)) and abs(im - rb) <= 1e-13 * max(1, abs(rb))
        assert abs(fre - ra) <= 1e-5 * max(1, abs(ra)) and abs(fim - rb) <= 1e-5 * max(1, abs(rb))


def test_dual_result_type(binary):
    """NT = gbint::dual<double/float> (the role of autodiff::real in the reference, e.g.
    DiFfRG/tests/physics/integration/integrator_1D_cartesian_gpu.cu:133-184): value and
    derivative components are reduced separately and equal the two plain FP64 integrals of
    e^{-s u} f and -u e^{-s u} f (FP64 to rounding, FP32 to 1e-5), for the angle, Cartesian 1D
    and finite-T q0 families, through get() and request()."""
    out = run(binary, [], extra=["--dual"])
    rows = [l.split()[1:] for l in out if l.startswith("DUAL")]
    assert len(rows) == 16
    fams = set()
    for fam, *vals in rows:
        v, d, pv, pd = map(float, vals)
        fams.add(fam)
        tol = 1e-5 if fam == "ANGLEF" else 1e-13
        assert abs(v - pv) <= tol * max(1, abs(pv)), (fam, v, pv)
        assert abs(d - pd) <= tol * max(1, abs(pd)), (fam, d, pd)
        assert abs(pd) > 1e-6  # the derivative is not trivially zero (integrals here are ~1e-4..1e-2)
    assert fams == {"ANGLE", "ANGLEF", "CART1", "FTQ0"}


def _reg_closed_forms(name, k2, q2):
    """RB, RBdot, dq2RB, RF, RFdot, dq2RF of the regulator shapes, written out in numpy
    (nan where the class does not define the function)."""
    x = q2 / k2
    nan = float("nan")
    if name == "litim":
        RB, RBdot, dRB = (k2 - q2) * (k2 > q2), 2 * k2 * (k2 > q2), nan
    elif name.startswith("bosonic"):
        b = float(name[-1])
        y = x ** b
        em = math.expm1(y)
        RB = q2 * x ** (b - 1) / em
        dRB = b * x ** (b - 1) * (em - y * math.exp(y)) / em ** 2
        RBdot = 2 * k2 * y * (em * (1 - b) + b * y * math.exp(y)) / em ** 2
    elif name.startswith("exp"):
        b = float(name[-1])
        y = x ** b
        RB, dRB, RBdot = k2 * math.exp(-y), -b * x ** (b - 1) * math.exp(-y), 2 * k2 * math.exp(-y) * (1 + b * y)
    elif name == "smoothlitim":
        a = 2e-3
        E = math.exp(min((x - 1) / a, 700.0))
        RB = (k2 - q2) / (1 + E)
        RBdot = 0.0 if E > 1e50 else 2 * k2 * (1 + E * (x - x * x + a) / a) / (1 + E) ** 2
        dRB = nan
    elif name.startswith("ratexp"):
        # f = P/D: D = 1 + b0 x^(n//2) + g x^(n-1), g = (1/n + b0/ceil(n/2))/(c-1), P = [D(x) (-ln(1-x))] up to x^n
        n = int(name[len("ratexp"):])
        c, b0 = (2.0, 0.0) if n == 8 else (1.5, 0.25)
        g = (1.0 / n + b0 / (n - n // 2)) / (c - 1)
        d = [0.0] * n
        d[0] += 1
        d[n // 2] += b0
        d[n - 1] += g
        pc = [0.0] + [sum(d[l] / (i - l) for l in range(min(i, n))) for i in range(1, n + 1)]
        D = sum(d[l] * x ** l for l in range(n))
        dD = sum(l * d[l] * x ** (l - 1) for l in range(1, n))
        P = sum(pc[i] * x ** i for i in range(1, n + 1))
        dP = sum(i * pc[i] * x ** (i - 1) for i in range(1, n + 1))
        f, fp = P / D, (dP * D - P * dD) / D ** 2
        RB, RBdot, dRB = k2 * math.exp(-f), 2 * k2 * math.exp(-f) * (1 + x * fp), -math.exp(-f) * fp
    else:
        n = int(name[len("polyexp"):])
        f = sum(x ** m / m for m in range(1, n + 1))
        fp = sum(x ** (m - 1) for m in range(1, n + 1))
        RB, RBdot, dRB = k2 * math.exp(-f), 2 * k2 * math.exp(-f) * (1 + x * fp), -math.exp(-f) * fp
    s = math.sqrt(RB + q2)
    RF, RFdot = s - math.sqrt(q2), 0.5 * RBdot / s
    dRF = (1 + dRB) / (2 * s) - 1 / (2 * math.sqrt(q2))
    return [RB, RBdot, dRB, RF, RFdot, dRF]


def test_regulators_host_device_and_derivatives(binary):
    """gbint/regulators.hh (the reference's regulator classes, DiFfRG/include/DiFfRG/physics/
    regulators.hh): every function on the host equals the device value and the numpy closed
    form, and the analytic derivatives equal forward differentiation with gbint::dual
    (dq2RB, dq2RF in q^2; RBdot, RFdot as 2 k^2 d/dk^2)."""
    out = run(binary, [], extra=["--regulators"])
    rows = [l.split()[1:] for l in out if l.startswith("REG")]
    names = {r[0] for r in rows}
    assert names == {"litim", "bosonic2", "bosonic1", "exp2", "exp3", "smoothlitim", "polyexp8", "polyexp3",
                     "ratexp8", "ratexp5"}
    checked_ad = 0
    for name, k2, q2, fn, host, dev, ad in rows:
        k2, q2, fn, host, dev, ad = float(k2), float(q2), int(fn), float(host), float(dev), float(ad)
        want = _reg_closed_forms(name, k2, q2)[fn]
        if math.isnan(want):
            assert math.isnan(host) and math.isnan(dev)
            continue
        # relative 1e-9: the shape formulas cancel near q^2 -> 0 (e.g. the bosonic dq2RB,
        # expm1(y) - y e^y ~ -y^2/2 at y = 1e-6 keeps ~9 digits); an absolute floor for values
        # formed by cancellation of O(1) terms (dq2RF where R_B is negligible)
        assert abs(host - want) <= 1e-9 * abs(want) + 1e-14, (name, k2, q2, fn, host, want)
        assert abs(dev - host) <= 1e-13 * abs(host) + 1e-15, (name, k2, q2, fn, dev, host)
        if not math.isnan(ad):
            assert abs(ad - host) <= 1e-9 * abs(host) + 1e-13, (name, k2, q2, fn, ad, host)
            checked_ad += 1
    assert checked_ad > 100


def test_fanout_helpers_equal_direct_gets(binary):
    """request_data / update_data / update_interpolator / get_data / make_grid (gbint/flow_utils.hh,
    the reference's DiFfRG/include/DiFfRG/physics/utils.hh:31-220) over a grid of external
    momenta, a 1D coordinates object (arguments as a tuple) and a 2D coordinate pack, and a
    RequestBatch scope mixing grids, k values, integral sizes, staged interpolator tables and a
    dual result type with a get() inside the scope: every batched value bit-identical to one get()
    per point."""
    out = run(binary, [], extra=["--fanout"])
    rows = {l.split()[1]: (float(l.split()[2]), int(l.split()[3])) for l in out if l.startswith("FAN")}
    assert set(rows) == {"request_data_vector", "request_data_coordinates_tuple", "get_data", "update_interpolator",
                         "request_data_pack2d", "request_batch_scope", "request_batch_scope_dual", "staging_fallbacks"}
    assert rows["staging_fallbacks"][0] == 0.0  # every launch read its staged arrays from shared memory
    for what, (diff, n) in rows.items():
        assert n > 0 and diff == 0.0, (what, diff, n)


def test_generated_style_kernel_through_cpu_class_name(binary):
    """A KERNEL written the way the reference's code generator writes them (regulator template,
    templated argument types, powr / complex / real from gbint/kernel_math.hh, private RB
    forwarding), through the CPU class name IntegratorFiniteTq0TBB (an alias of the GPU class),
    equals the same integrand in plain real arithmetic to rounding."""
    out = run(binary, [], extra=["--generated"])
    rows = [list(map(float, l.split()[1:])) for l in out if l.startswith("GEN")]
    assert len(rows) == 4
    for T, gen, plain in rows:
        assert abs(gen - plain) <= 1e-13 * abs(plain), (T, gen, plain)
        assert abs(plain) > 1e-6
