"""GPU: the quasi-Monte-Carlo integrators (include/gbint/qmc.hh) -- IntegratorQMC<d>,
IntegratorAngleQMC<d>, Integrator4DQMC -- on the reference's own test cases
(DiFfRG/tests/physics/integration/integrator{,_angle,_4D}_qmc.cc): volume integrals and random
polynomials against their closed forms.

The reference's QMC results are random (its shifts come from std::random_device), so parity is
statistical, as in its tests: each value must meet the reference's tolerance (1e-2 for the 1D
volume with its 1/q singularity, 1e-6 for the other volumes, 2e-2 for random polynomials) and,
tighter, lie within 6 standard errors of the exact value with the error estimate meeting the
requested tolerance unless the evaluation budget ran out.
"""
import subprocess

import pytest

pytestmark = pytest.mark.gpu

# (reference tolerance, requested rel_tol, maxeval) per case
CASES = {
    "QMC1_volume": (1e-2, 1e-6, 2000000), "QMC2_volume": (1e-6, 1e-6, 2000000),
    "QMC3_volume": (1e-6, 1e-6, 2000000), "QMC4_volume": (1e-6, 1e-6, 2000000),
    "QMC1_poly": (2e-2, 1e-4, 500000), "QMC2_poly": (2e-2, 1e-4, 500000), "QMC3_poly": (2e-2, 1e-4, 500000),
    "QMC4_poly": (2e-2, 1e-4, 500000), "AngleQMC2_poly": (2e-2, 1e-4, 1000000),
    "AngleQMC3_poly": (2e-2, 1e-4, 1000000), "AngleQMC4_poly": (2e-2, 1e-4, 1000000),
    "4DQMC_volume": (1e-6, 1e-4, 500000), "4DQMC_poly": (2e-2, 1e-4, 500000),
}


def is_close(a, b, eps):
    """DiFfRG/include/DiFfRG/common/math.hh:160-172 (absolute or relative)."""
    d = abs(a - b)
    return d <= eps or d <= max(abs(a), abs(b)) * eps


@pytest.fixture(scope="module")
def results():
    from diffrg_gb300 import cppapi

    exe = cppapi.build_qmc_tests()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {}
    for ln in r.stdout.strip().splitlines():
        f = ln.split()
        out[f[0]] = dict(value=float(f[1]), exact=float(f[2]), error=float(f[3]), n=int(f[4]), m=int(f[5]),
                         evals=int(f[6]))
    return out


@pytest.mark.parametrize("case", sorted(CASES))
def test_qmc_case(results, case):
    tol, rel, maxeval = CASES[case]
    r = results[case]
    assert is_close(r["exact"], r["value"], tol), r
    if case != "QMC1_volume":  # 1/sqrt(x) in the unit cube: infinite variance, the estimate is no bound
        assert abs(r["value"] - r["exact"]) <= max(6 * r["error"], 1e-14 * abs(r["exact"])), r
    if r["evals"] < maxeval:  # converged: the estimate meets the requested tolerance
        assert r["error"] <= max(1e-16, rel * abs(r["value"])) * 1.000001, r
    assert r["m"] >= 32 and r["n"] >= 1021
