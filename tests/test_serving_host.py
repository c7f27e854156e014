"""Host logic of the C4 serving driver (no GPU): the Cash-Karp pair, the adaptive stepper,
the request-size stream and the gb_integral layout the request loop receives."""
import ctypes as C
import math

import numpy as np
import pytest

from diffrg_gb300 import serving as S
from diffrg_gb300.capi import Integral


def test_cash_karp_tableau_order_conditions():
    c, A, b5, b4 = S.CK_C, S.CK_A, np.array(S.CK_B5), np.array(S.CK_B4)
    for s in range(6):
        assert abs(sum(A[s]) - c[s]) < 1e-15
    cc = np.array(c)
    # order conditions up to 4 (both weights) and 5 (b5): sum b c^(q-1) = 1/q
    for q in range(1, 5):
        assert abs(np.dot(b4, cc ** (q - 1)) - 1 / q) < 1e-14, q
    for q in range(1, 6):
        assert abs(np.dot(b5, cc ** (q - 1)) - 1 / q) < 1e-14, q


@pytest.mark.parametrize("h", [0.2, 0.1])
def test_cash_karp_step_is_fifth_order(h):
    y5, err = S.cash_karp_step(lambda t, y: -y, 0.0, np.array([1.0]), h)
    assert abs(y5[0] - math.exp(-h)) < 2e-3 * h ** 6
    assert abs(err[0]) < 1e-2 * h ** 5 + 1e-16


def test_adaptive_integration_reaches_tolerance():
    y, acc, rej = S.integrate_adaptive(lambda t, y: np.cos(t) * y, np.array([1.0, 2.0]), 0.0, 3.0, h0=0.5,
                                       rtol=1e-10, atol=1e-12)
    exact = np.exp(np.sin(3.0)) * np.array([1.0, 2.0])
    assert np.max(np.abs(y - exact) / exact) < 1e-8
    assert acc > 5


def test_request_sizes_cover_the_rhs():
    rng = np.random.default_rng(5)
    for total in (4096, 100, 8, 3000):
        sz = S.request_sizes(rng, total, 8, 2048)
        assert sum(sz) == total
        assert max(sz) <= 2048
        assert all(s >= 1 for s in sz)
        assert all(s >= 8 for s in sz[:-1]) or total < 16


def test_c4_workload_shape():
    w = S.c4()
    assert len(w["funcs"]) == 32 and w["y0"].shape == (32, 128)
    for f in w["funcs"]:
        assert len(f["orders"]) == f["dim"] and all(32 <= n <= 128 for n in f["orders"])
    items = S.rhs_items(w, 0.5)
    assert len(items) == 4096
    tl = S.table_order()
    for i, f in enumerate(w["funcs"]):
        g = items[i * 128]
        assert g.table_base == i
        if f["dim"] == 3:  # four contiguous entries naming tables i..i+3 (cyclic)
            assert [tl[g.table_base + m] for m in range(4)] == [(i + m) % 32 for m in range(4)]


def test_integral_layout_keeps_the_field_offsets():
    """table_base fills the padding after n[4]: the other fields keep their offsets."""
    assert Integral.table_base.offset == 28
    assert Integral.x_extent.offset == 32
    assert C.sizeof(Integral) == 320 and Integral.args.offset == 128
