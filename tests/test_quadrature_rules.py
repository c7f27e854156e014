"""The rules of every QuadratureType (QuadratureProvider::get_points/get_weights with a type;
DiFfRG/include/DiFfRG/common/quadrature/quadrature.hh:47, quadrature.cu:12-60: GSL's fixed
types with a = 0, b = 1, alpha = beta = 0) -- CPU, through the host-only C entry
gb_quad_rule_host (no context, no GPU).

References: Chebyshev nodes and weights in closed form (and numpy's chebgauss); Laguerre and
Hermite nodes refined by Newton's method and weights from their closed forms, both in 80-digit
mpmath; Jacobi(0,0) is the Legendre rule bit for bit; moments of the weight functions.
"""
import math

import numpy as np
import pytest

from diffrg_gb300 import engine as E
from diffrg_gb300.capi import GbError

mp = pytest.importorskip("mpmath")


def _lag(n, z):
    p0, p1 = mp.mpf(1), 1 - z
    if n == 0:
        return p0, mp.mpf(0)
    for k in range(1, n):
        p0, p1 = p1, ((2 * k + 1 - z) * p1 - k * p0) / (k + 1)
    return p1, p0


def _her(n, z):
    p0, p1 = mp.mpf(1), 2 * z
    if n == 0:
        return p0, mp.mpf(0)
    for k in range(1, n):
        p0, p1 = p1, 2 * z * p1 - 2 * k * p0
    return p1, p0


@pytest.mark.parametrize("n", [1, 2, 5, 16, 64, 100])
def test_laguerre_rule_to_full_relative_precision(n):
    mp.mp.dps = 80
    x, w = E.quad_rule_host(E.QUAD_LAGUERRE, n)
    assert np.all(np.diff(x) > 0)
    for xi, wi in zip(x, w):
        z = mp.mpf(xi)
        for _ in range(4):
            ln, ln1 = _lag(n, z)
            z = z - ln / (n * (ln - ln1) / z)
        wt = z / ((n + 1) ** 2 * _lag(n + 1, z)[0] ** 2)
        assert abs(float((mp.mpf(xi) - z) / z)) <= 4e-16
        assert abs(float((mp.mpf(wi) - wt) / wt)) <= 4e-16, (n, xi, wi)
    # tail weights keep full relative precision (n = 100: down to ~3e-162)
    assert w.sum() == pytest.approx(1.0, rel=1e-15, abs=0)


@pytest.mark.parametrize("n", [1, 2, 5, 16, 64, 200])
def test_hermite_rule_to_full_relative_precision(n):
    mp.mp.dps = 80
    x, w = E.quad_rule_host(E.QUAD_HERMITE, n)
    assert np.all(np.diff(x) > 0)
    assert np.array_equal(x, -x[::-1]) and np.allclose(w, w[::-1], rtol=1e-15, atol=0)
    for xi, wi in zip(x, w):
        z = mp.mpf(xi)
        if n % 2 == 0 or xi != 0.0:
            for _ in range(4):
                hn, hn1 = _her(n, z)
                z = z - hn / (2 * n * hn1)
        wt = 2 ** (n - 1) * mp.factorial(n) * mp.sqrt(mp.pi) / (n ** 2 * _her(n - 1, z)[0] ** 2)
        assert abs(float(mp.mpf(xi) - z)) <= 4e-16 * max(1.0, abs(xi))
        assert abs(float((mp.mpf(wi) - wt) / wt)) <= 4e-16, (n, xi, wi)
    assert w.sum() == pytest.approx(math.sqrt(math.pi), rel=1e-15)


def test_laguerre_weights_below_the_fp64_range_are_zero():
    x, w = E.quad_rule_host(E.QUAD_LAGUERRE, 200)
    assert np.all(w >= 0) and np.all(np.isfinite(w)) and np.all(np.isfinite(x))
    assert w.sum() == pytest.approx(1.0, rel=1e-15)


@pytest.mark.parametrize("n", [1, 3, 8, 33, 128])
def test_chebyshev_rule_closed_form(n):
    x, w = E.quad_rule_host(E.QUAD_CHEBYSHEV, n)
    t = (2 * np.arange(n) + 1) * math.pi / (2 * n)
    np.testing.assert_allclose(x, np.sin(t / 2) ** 2, rtol=0, atol=4.5e-16)  # the FP64 reference is ~2 ulp
    assert np.all(w == w[0]) and w[0] == pytest.approx(math.pi / n, rel=1e-16)
    xc, wc = np.polynomial.chebyshev.chebgauss(n)
    np.testing.assert_allclose(x, np.sort((1 + xc) / 2), rtol=0, atol=4.5e-16)
    # int_0^1 x^k / sqrt(x (1-x)) dx = pi (2k-1)!! / (2k)!! = pi C(2k, k) / 4^k, exact for k < 2n
    for k in range(0, 2 * n, max(1, n // 4)):
        exact = math.pi * (math.comb(2 * k, k) / 4 ** k)
        assert np.sum(w * x ** k) == pytest.approx(exact, rel=1e-13)


@pytest.mark.parametrize("n", [1, 4, 17, 64, 300])
def test_jacobi_is_the_legendre_rule(n):
    xj, wj = E.quad_rule_host(E.QUAD_JACOBI, n)
    xl, wl = E.quad_rule_host(E.QUAD_LEGENDRE, n)
    assert np.array_equal(xj, xl) and np.array_equal(wj, wl)
    assert wl.sum() == pytest.approx(1.0, rel=1e-14)


def test_moments_of_laguerre_and_hermite():
    n = 12
    x, w = E.quad_rule_host(E.QUAD_LAGUERRE, n)
    for k in range(2 * n):
        assert np.sum(w * x ** k) == pytest.approx(math.factorial(k), rel=1e-12)
    x, w = E.quad_rule_host(E.QUAD_HERMITE, n)
    for k in range(0, 2 * n, 2):
        assert np.sum(w * x ** k) == pytest.approx(math.gamma((k + 1) / 2), rel=1e-12)


@pytest.mark.parametrize("qtype,order", [(5, 4), (-1, 4), (2, 0), (3, 5000)])
def test_bad_type_or_order_is_an_error(qtype, order):
    with pytest.raises(GbError):
        E.quad_rule_host(qtype, order)
