"""Oracle pinning: every integrator family against the analytic integrals of the polynomial KERNEL,
as the reference's integrator tests do (volume integrals and random polynomials)."""
import math

import numpy as np
import pytest

from kat import CASES, analytic, random_args

# analytic-vs-quadrature tolerances; the reference uses 1e-6 (volume) and 1e-4 (polynomials)
TOL = {"FTQ0": 5e-5, "ANGLE_FTQ0": 5e-5, "4D_FTQ0": 5e-5}


def family_inputs(fam, seed):
    rng = np.random.default_rng(seed)
    kw = dict(CASES[fam])
    n = kw.pop("n")
    d = kw.pop("d")
    k = rng.uniform(0.3, 1.0)
    xe = rng.uniform(1.0, 2.0)
    T = kw.get("T", 0.0)
    if fam.endswith("FTQ0"):
        args = random_args(rng, q0_rational=(T, rng.uniform(0.8, 1.2)))
    else:
        args = random_args(rng)
    if fam.endswith("FTX0"):
        ns = kw["x0_summands"]
        kw["x0_extent"] = ns * 10 * 2 * math.pi * T / k * 1.5 + 1000.0 / k
    return n, d, k, xe, args, kw


def oracle_family(O, fam, n, d, k, xe, args, kw):
    E = O.resolve_E(kw.get("T", 0.0), k) if fam.endswith("FTQ0") else 0.0
    desc = O.family_desc(fam, d=d, n=n, x_extent=xe, x0_extent=kw.get("x0_extent", 0.0),
                         x0_summands=kw.get("x0_summands", 0), T=kw.get("T", 0.0), E=E,
                         qmin=kw.get("qmin", (-math.pi,) * 3), qmax=kw.get("qmax", (math.pi,) * 3))
    return O.family(desc, "POLY", k, args[None, :])[0]


@pytest.mark.parametrize("fam", list(CASES))
@pytest.mark.parametrize("seed", [1, 2])
def test_family_random_polynomials(oracle, fam, seed):
    n, d, k, xe, args, kw = family_inputs(fam, seed)
    got = oracle_family(oracle, fam, n, d, k, xe, args, kw)
    ref = analytic(fam, args, k, d=d, x_extent=xe, **kw)
    tol = TOL.get(fam, 1e-4)
    assert math.isfinite(got)
    assert abs(got - ref) <= tol * max(1.0, abs(ref)), (fam, got, ref)


@pytest.mark.parametrize("fam", ["1D", "ANGLE", "3D", "4D2ANG", "4D"])
def test_family_volume(oracle, fam):
    """Volume integral V_d(q_ext)/(2 pi)^d at 1e-6 (integrator_4D_gpu.cu:48-62)."""
    n, d, k, xe, args, kw = family_inputs(fam, 7)
    a = np.zeros(24)
    a[1] = 1.0
    a[7] = a[11] = a[15] = a[19] = 1.0
    if fam in ("4D2ANG", "4D"):
        a[7:11] = [1, 0, 0, 0]  # the cos1 Jacobian is part of the measure
    got = oracle_family(oracle, fam, n, d, k, xe, a, kw)
    ref = analytic(fam, a, k, d=d, x_extent=xe, **kw)
    qe = math.sqrt(xe) * k
    dim = {"3D": 3}.get(fam, d)
    vol = math.pi ** (dim / 2) / math.gamma(dim / 2 + 1) * qe ** dim / (2 * math.pi) ** dim
    assert abs(ref - vol) <= 1e-12 * vol
    # the sqrt(1-cos1^2) Jacobian limits Gauss-Legendre to algebraic convergence in the cos1 order
    tol = 5e-4 if fam in ("4D2ANG", "4D") else 1e-6
    assert abs(got - vol) <= tol * vol


def test_finiteTx0_volume(oracle):
    """integrator_finiteTx0_gpu.cu:53-70: spatial volume x [(2N_s - 1) T + (q0_ext - 2 pi T N_s) 2/(2 pi)]."""
    T, k, xe, ns = 0.3, 0.7, 1.5, 32
    x0e = ns * 10 * 2 * math.pi * T / k * 1.4 + 1000.0 / k
    a = np.zeros(24)
    a[1] = 1.0
    a[19] = 1.0
    desc = oracle.family_desc("FTX0", d=4, n=(64, 64), x_extent=xe, x0_extent=x0e, x0_summands=ns, T=T)
    got = oracle.family(desc, "POLY", k, a[None, :])[0]
    qe = math.sqrt(xe) * k
    vol3 = 4 / 3 * math.pi * qe ** 3 / (2 * math.pi) ** 3
    ref = vol3 * ((2 * ns - 1) * T + (x0e * k - 2 * math.pi * T * ns) * 2 / (2 * math.pi))
    assert abs(got - ref) <= 5e-5 * ref


def test_oracle_is_deterministic_across_threads(oracle):
    n, d, k, xe, args, kw = family_inputs("4D", 3)
    desc = oracle.family_desc("4D", d=d, n=n, x_extent=xe)
    A = np.tile(args, (8, 1))
    a1 = oracle.family(desc, "POLY", k, A, threads=1)
    a4 = oracle.family(desc, "POLY", k, A, threads=4)
    assert np.array_equal(a1, a4)
