"""gb_get_noalloc: the allocation-free FP64 entry point for hosts that may not allocate device
memory while integrating (e.g. under CUDA stream capture in global mode, or under a fixed
memory budget owned by another allocator).  Its scratch is a fixed device array inside the
library, so every call reuses the previous call's memory: the test calls it twice in a row per
integral and compares both results with gb_get in FP64 through the C ABI.

This file is named to be collected last, so that a failure here cannot hide other tests.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12  # the tolerance the FP64 parity tests use


def _get_noalloc(ctx, g, tables=()):
    from diffrg_gb300 import capi
    from diffrg_gb300.engine import _table_array

    out = C.c_double()
    rc = capi.lib().gb_get_noalloc(ctx.h, C.byref(g), _table_array(tables), len(tables), C.byref(out))
    return rc, out.value


def test_noalloc_matches_gb_get_twice_in_a_row():
    from diffrg_gb300 import workloads as W
    from diffrg_gb300.engine import Context, integral
    from kat import random_args

    rng = np.random.default_rng(21)
    ctx = Context(0)
    try:
        cases = []
        cases.append((integral("4D", "POLY", n=(64, 16, 12, 8), k=0.7, x_extent=1.5, args=random_args(rng)), ()))
        cases.append((integral("ANGLE_FTQ0", "POLY", n=(48, 12), k=0.6, T=0.2, x_extent=1.2,
                               args=random_args(rng, q0_rational=(0.2, 1.1))), ()))
        k = 0.8
        cases.append((integral("FTX0", "POLY", n=(64, 48), k=k, T=0.3, x_extent=1.3, x0_summands=16,
                               x0_extent=16 * 10 * 2 * math.pi * 0.3 / k + 1000 / k, args=random_args(rng)), ()))
        w = W.c3(64)
        items, tabs = W.engine_items(w)
        T3 = [ctx.table(s, d) for s, d in tabs]
        keep = [i for i in range(64) if int(np.prod(w["orders"][i].astype(np.int64))) <= 2_000_000][:3]
        cases += [(items[i], T3) for i in keep]
        w5 = W.c5()
        items5, tabs5 = W.engine_items(w5)
        T5 = [ctx.table(s, d) for s, d in tabs5]
        small = integral("4D", "VERT4", n=(64, 16, 8, 8), k=1.0, x_extent=4.0, args=items5[7].args[:4])
        cases.append((small, T5))
        for g, tables in cases:
            ref = ctx.get(g, tables, "fp64")
            rc1, v1 = _get_noalloc(ctx, g, tables)
            rc2, v2 = _get_noalloc(ctx, g, tables)
            assert rc1 == 0 and rc2 == 0, ctx.last_error()
            assert abs(v1 - ref) <= TOL64 * abs(ref)
            assert abs(v2 - ref) <= TOL64 * abs(ref)
    finally:
        ctx.close()


def test_noalloc_rejects_integrals_beyond_its_scratch():
    from diffrg_gb300.engine import Context, integral

    ctx = Context(0)
    try:
        big = integral("4D", "POLY", n=(128, 64, 32, 32), k=1.0, args=(0, 1))  # 8.4M grid points
        rc, _ = _get_noalloc(ctx, big)
        assert rc == 1
        assert "at most 4194304" in ctx.last_error()
    finally:
        ctx.close()
