"""CPU: the per-cell propagator series that C3's kernel reads for its table B.

`k_cell_records` (diffrg_gb300/csrc/kernels_generic.cu) expands 1 / (Z(x) x + R(x)) about each
cell centre c_j of a log table in t = x / c_j - 1, through t^8: Z is the cell's linear segment in
the log index, z0 + z1 ln(1 + t), R(x) = x / expm1(x) the regulator, and the coefficients come
from a series reciprocal in FP64.  A cell is trusted when the tail estimated from the last two
coefficients stays below 1e-12 of g0; other cells are evaluated from the value record and the
regulator.  This restates that construction in numpy and checks what the kernel relies on: a
trusted cell's series is exact to ~1e-11 everywhere in its cell (FP64 coefficients, so the
kernel's FP32 tail g3..g8 adds only its own rounding), nearly every cell of the benchmark tables
is trusted, and on a table whose value jumps 60 % between cells the test refuses a large share.
"""
import math

import numpy as np

from diffrg_gb300 import workloads as W

N_TAB, LO, HI = 256, 1e-4, 100.0
SCALE = (N_TAB - 1) / math.log2(HI / LO)
SHIFT = -math.log2(LO) * SCALE
K = 9  # coefficients g0..g8


def _regulator_coeffs(c):
    """Taylor coefficients of R(c (1 + t)) = c (1 + t) / expm1(c (1 + t)) in t."""
    d = [math.expm1(c)] + [math.exp(c) * c ** k / math.factorial(k) for k in range(1, K)]
    a = []
    for k in range(K):
        nk = c if k < 2 else 0.0
        for i in range(k):
            nk -= a[i] * d[k - i]
        a.append(nk / d[0])
    return a


def _cell_series(y, j):
    c = 2.0 ** ((j + 0.5 - SHIFT) / SCALE)
    d = float(y[j + 1]) - float(y[j])
    z0, z1 = float(y[j]) + 0.5 * d, d * SCALE / math.log(2.0)
    w = [z0] + [z1 * (1.0 if k % 2 else -1.0) / k for k in range(1, K)]
    a = _regulator_coeffs(c)
    D = [c * w[0] + a[0]] + [c * (w[k] + w[k - 1]) + a[k] for k in range(1, K)]
    g = [1.0 / D[0]]
    for k in range(1, K):
        g.append(-g[0] * sum(D[i] * g[k - i] for i in range(1, k + 1)))
    h = math.expm1(math.log(2.0) / (2.0 * SCALE))  # the cell spans |t| <= h
    rt = abs(g[-1] / g[-2]) * h if g[-2] != 0 else 1.0
    trusted = D[0] > 0 and rt < 0.5 and abs(g[-1]) * h ** (K - 1) * rt / (1 - rt) <= 1e-12 * abs(g[0])
    return c, g, trusted


def _exact(y, x):
    u = min(max(SCALE * math.log2(x) + SHIFT, 0.0), N_TAB - 1.0)
    i = min(int(u), N_TAB - 2)
    z = float(y[i]) + (u - i) * (float(y[i + 1]) - float(y[i]))
    return 1.0 / (z * x + x / math.expm1(x))


def _check_table(y, rng):
    """(cells trusted, worst relative error of the series over the trusted cells)."""
    trusted_cells, worst = 0, 0.0
    for j in range(N_TAB - 1):
        c, g, trusted = _cell_series(y, j)
        if not trusted:
            continue
        trusted_cells += 1
        for s in list(rng.uniform(-0.5, 0.5, 6)) + [-0.4999999, 0.4999999]:
            x = 2.0 ** ((j + 0.5 + s - SHIFT) / SCALE)
            t = x / c - 1.0
            series = sum(gk * t ** k for k, gk in enumerate(g))
            worst = max(worst, abs(series / _exact(y, x) - 1.0))
    return trusted_cells, worst


def test_trusted_cells_are_exact_on_the_benchmark_tables():
    rng = np.random.default_rng(4)
    for _, y in W.c3()["tables"]:
        trusted, worst = _check_table(y, rng)
        assert trusted >= 0.95 * (N_TAB - 1), trusted  # the rest take the value record + regulator
        assert worst <= 1e-11, worst


def test_steep_table_cells_are_refused():
    rng = np.random.default_rng(5)
    y = np.where(np.arange(N_TAB) % 2 == 0, 0.4, 1.0).astype(np.float32)
    trusted, worst = _check_table(y, rng)
    assert trusted <= 0.6 * (N_TAB - 1), trusted
    assert worst <= 1e-11, worst
