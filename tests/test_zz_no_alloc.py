"""gb_get_noalloc: the allocation-free FP64 entry point.

It exists for callers that cannot let the library allocate device memory while they integrate:
a program whose HBM already belongs to another allocator (a caching or pool allocator that
reserved it at start-up, or a fixed budget granted once) and callers that cannot take the
device-wide wait of cudaFree.  Its scratch is a fixed device array inside the library, so every
call finds the previous call's contents there: the tests call it twice in a row per integral
and compare both results with gb_get (the allocating entry point) through the C ABI, and the
polynomial cases also with the FP64 oracle.  A third test checks that a run of calls with new
RG scales and new quadrature orders leaves the device's free memory unchanged, a fourth that a
call made while another stream captures a CUDA graph (relaxed mode) runs eagerly and leaves the
capture valid.

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


def _poly_cases(rng):
    """(family, n, d, k, x_extent, args, kw) of POLY integrals the oracle also evaluates."""
    from kat import random_args

    k = 0.8
    return [
        ("4D", (64, 16, 12, 8), 4, 0.7, 1.5, random_args(rng), {}),
        ("ANGLE_FTQ0", (48, 12), 4, 0.6, 1.2, random_args(rng, q0_rational=(0.2, 1.1)), {"T": 0.2}),
        ("FTX0", (64, 48), 4, k, 1.3, random_args(rng),
         {"T": 0.3, "x0_summands": 16, "x0_extent": 16 * 10 * 2 * math.pi * 0.3 / k + 1000 / k}),
    ]


def _engine_integral(fam, n, d, k, xe, args, kw):
    from diffrg_gb300.engine import integral

    return integral(fam, "POLY", n=n, d=d, k=k, x_extent=xe, args=args, **kw)


def test_noalloc_matches_gb_get_twice_in_a_row(oracle):
    from diffrg_gb300 import workloads as W
    from diffrg_gb300.engine import Context, integral
    from test_oracle_families import oracle_family

    rng = np.random.default_rng(21)
    ctx = Context(0)
    try:
        cases = []
        for fam, n, d, k, xe, args, kw in _poly_cases(rng):
            want = oracle_family(oracle, fam, n, d, k, xe, args, kw)
            cases.append((_engine_integral(fam, n, d, k, xe, args, kw), (), want))
        w = W.c3(64)
        items, tabs = W.engine_items(w)
        T3 = [ctx.table(s, d) for s, d in tabs]
        keep = [i for i in range(64) if int(np.prod(w["orders"][i].astype(np.int64))) <= 2_000_000][:3]
        cases += [(items[i], T3, None) for i in keep]
        w5 = W.c5()
        items5, tabs5 = W.engine_items(w5)
        T5 = [ctx.table(s, d) for s, d in tabs5]
        small = integral("4D", "VERT4", n=(64, 16, 8, 8), k=1.0, x_extent=4.0, args=items5[7].args[:4])
        cases.append((small, T5, None))
        for g, tables, want in cases:
            ref = ctx.get(g, tables, "fp64")
            rc1, v1 = _get_noalloc(ctx, g, tables)
            rc2, v2 = _get_noalloc(ctx, g, tables)
            assert rc1 == 0 and rc2 == 0, ctx.last_error()
            assert abs(v1 - ref) <= TOL64 * abs(ref)
            assert abs(v2 - ref) <= TOL64 * abs(ref)
            if want is not None:  # the oracle's FP64 restatement of the reference CPU integrator
                assert abs(v1 - want) <= TOL64 * max(1.0, abs(want)), (v1, want)
    finally:
        ctx.close()


def test_noalloc_leaves_free_device_memory_unchanged():
    """New RG scales k (each builds a new radial axis) and new orders go into the node pool that
    gb_ctx_create reserved; nothing is allocated, so cudaMemGetInfo's free bytes do not move."""
    import torch

    from diffrg_gb300.engine import Context

    rng = np.random.default_rng(5)
    ctx = Context(0)
    try:
        fam, n, d, k, xe, args, kw = _poly_cases(rng)[0]
        for _ in range(2):  # first call per device: address look-up, module load
            rc, _ = _get_noalloc(ctx, _engine_integral(fam, n, d, k, xe, args, kw))
            assert rc == 0, ctx.last_error()
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info(0)
        got = []
        for i in range(12):
            kk = 0.5 + 0.037 * i                     # a new radial axis every call
            nn = (32 + 4 * i, 8 + i, 6 + (i % 5), 8)  # new orders on every axis
            g = _engine_integral(fam, nn, d, kk, xe, args, kw)
            rc, v = _get_noalloc(ctx, g)
            assert rc == 0, ctx.last_error()
            got.append((nn, kk, v))
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info(0)
        assert free1 == free0, (free0, free1)
        for nn, kk, v in got:  # gb_get allocates, so it runs after the window
            ref = ctx.get(_engine_integral(fam, nn, d, kk, xe, args, kw), (), "fp64")
            assert abs(v - ref) <= TOL64 * abs(ref)
    finally:
        ctx.close()


def test_noalloc_runs_eagerly_while_a_relaxed_capture_is_open():
    """A call made while this thread records a CUDA graph on another stream in relaxed capture
    mode (the integral's axes used once before) runs at once on the context's stream and is not
    recorded: it returns the same value as before the capture, the capture stays valid, and its
    replays run only the captured work.  (In global or thread-local mode the call's stream wait
    is a prohibited call and invalidates the capture -- the header says so.)"""
    import torch

    from diffrg_gb300.engine import Context

    rng = np.random.default_rng(9)
    ctx = Context(0)
    try:
        fam, n, d, k, xe, args, kw = _poly_cases(rng)[0]
        g = _engine_integral(fam, n, d, k, xe, args, kw)
        rc, before = _get_noalloc(ctx, g)
        assert rc == 0, ctx.last_error()
        x = torch.zeros(4, device="cuda")
        graph = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            graph.capture_begin(capture_error_mode="relaxed")
            x.add_(1.0)
            rc, during = _get_noalloc(ctx, g)
            graph.capture_end()
        torch.cuda.current_stream().wait_stream(s)
        assert rc == 0, ctx.last_error()
        assert during == before
        graph.replay()
        graph.replay()
        torch.cuda.synchronize()
        assert x.tolist() == [2.0] * 4
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
