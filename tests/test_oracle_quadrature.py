"""Oracle pinning: quadrature rules against the reference's own golden tables and closed forms.

Mirrors DiFfRG/tests/common/quadrature/test_quadrature.cc:10-33 (make_quadrature vs the
constexpr GLQuadrature tables) and test_matsubara.cc:9-60 (Matsubara sums vs closed forms).
"""
import json
import math
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "gl_tables.json")


def gold_tables():
    d = json.load(open(GOLD))
    return {int(n): (np.array([float(v) for v in t["x"]]), np.array([float(v) for v in t["w"]]))
            for n, t in d["tables"].items()}


@pytest.mark.parametrize("n", [4, 8, 16, 32, 64, 128])
def test_gl_matches_reference_tables(oracle, n):
    x, w = oracle.gauss_legendre(n)
    gx, gw = gold_tables()[n]
    assert np.max(np.abs(x - gx)) < 1e-15
    assert np.max(np.abs(w - gw)) < 1e-15


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 100, 256, 512])
def test_gl_matches_numpy(oracle, n):
    x, w = oracle.gauss_legendre(n)
    xr, wr = np.polynomial.legendre.leggauss(n)
    assert np.max(np.abs(x - (xr + 1) / 2)) < 1e-14
    assert np.max(np.abs(w - wr / 2)) < 1e-13
    assert abs(w.sum() - 1) < 1e-14
    # exact for polynomials of degree 2n-1
    for deg in (0, n, 2 * n - 1):
        assert abs(np.sum(w * x ** deg) - 1.0 / (deg + 1)) < 1e-13


@pytest.mark.parametrize("n", [4, 8, 16, 32, 64, 128])
def test_golub_welsch_legendre_jacobi_matrix(oracle, n):
    """test_quadrature.cc: Jacobi matrix b_i = i^2/(4 i^2 - 1), mu0 = 2 reproduces GL on [-1,1]."""
    i = np.arange(1, n + 1, dtype=np.float64)
    b = i * i / (4 * i * i - 1)
    x, w = oracle.golub_welsch(np.zeros(n), b, 2.0)
    gx, gw = gold_tables()[n]
    assert abs(x[-1] - (2 * gx[-1] - 1)) < 1e-14
    assert abs(w[-1] - 2 * gw[-1]) < 1e-14
    assert np.max(np.abs(x - (2 * gx - 1))) < 1e-13
    assert np.max(np.abs(w - 2 * gw)) < 1e-13


@pytest.mark.parametrize("T", [0.0123, 0.05, 0.2, 0.5, 0.99])
def test_matsubara_coth(oracle, T):
    """test_matsubara.cc:11-23: T sum_n 1/(1+w_n^2) = coth(1/(2T))/2 at 1e-13."""
    s = oracle.matsubara_sum(lambda x: 1.0 / (1.0 + x * x), T, 1.0)
    ref = 0.5 / math.tanh(0.5 / T)
    assert abs(s - ref) <= 1e-13 * abs(ref)


@pytest.mark.parametrize("T,a,b", [(0.001, 0.1, 0.01), (0.01, 0.5, 0.05), (0.05, 1.0, 0.1), (0.1, 0.3, 0.02)])
def test_matsubara_shifted(oracle, T, a, b):
    """test_matsubara.cc:24-43: sum of 1/(a^2 + b w + w^2)."""
    s = oracle.matsubara_sum(lambda x: 1.0 / (a * a + b * x + x * x), T, a)
    r = math.sqrt(4 * a * a - b * b)
    ref = -(math.sinh(r / (2 * T)) / (r * (math.cos(b / (2 * T)) - math.cosh(r / (2 * T)))))
    assert abs(s - ref) <= 1e-13 * abs(ref)


@pytest.mark.parametrize("a", [0.01, 0.3, 1.0, 4.0, 10.0])
def test_matsubara_T0(oracle, a):
    """test_matsubara.cc:44-59: vacuum rule, integral 1/(a^2+w^2) dw/(2 pi) = 1/(2a) at 3e-6."""
    s = oracle.matsubara_sum(lambda x: 1.0 / (a * a + x * x), 0.0, a)
    assert abs(s - 1 / (2 * a)) <= 3e-6 / (2 * a)


def test_matsubara_size_prediction(oracle):
    """predict_size (matsubara.cu:12-20) and clamping to [min, max] with step 2."""
    for T, E in [(0.1, 1.0), (0.01, 1.0), (1.0, 1.0), (0.5, 0.2)]:
        x, w, tu = oracle.matsubara(T, E, step=2, min_size=0, max_size=1024)
        Emax = 101 * E
        size = 5 + int(math.sqrt(4 * Emax / (math.pi ** 2 * T)))
        size = int(math.ceil(size / 2) * 2)
        assert len(x) == size and tu == T
    x, w, tu = oracle.matsubara(0.001, 1.0, min_size=16, max_size=128)  # E/T > 100 -> vacuum
    assert tu == 0.0 and len(x) == 48
    x, w, tu = oracle.matsubara(0.5, 1.0, min_size=32, max_size=128)
    assert len(x) == 32
