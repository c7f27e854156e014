"""GPU: the device-resident request loop (gb_serve_start_device, dloop.cu).

gb_submit writes requests straight into a ring a persistent kernel reads; the kernel claims
published work units as CTAs free up and leaves after a bounded idle spin.
* results equal gb_get(..., FP64) to rounding (1e-14: the same per-point function and reduction
  order, compiled into another kernel) and the FP64 oracle within 1e-12, and are bit-identical
  alone and in a mix of concurrent requests submitted from several host threads;
* a request reads one table epoch (table updates wait for published requests);
* admission: a request that can never fit a ring slot is refused with GB_EBUDGET, a ring of two
  slots takes many requests in turn;
* the loop left alone runs dry: every CTA counts an idle exit, the kernel ends, and the next
  submit relaunches it cleanly with correct results;
* latency is stamped when a request finishes, not when it is waited for;
* a small request submitted behind a large one overtakes it (express lane).
"""
import threading
import time

import numpy as np
import pytest

from diffrg_gb300 import capi, serving
from diffrg_gb300.capi import GbError
from diffrg_gb300.engine import Context, integral

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def w():
    return serving.c4()


def _tables(c, w):
    ts = [c.table(w["spec"], w["y0"][i]) for i in range(serving.N_FUNC)]
    return ts, [ts[i] for i in serving.table_order()]


def _close(a, b, tol=1e-14):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.all(np.abs(a - b) <= tol * np.abs(b))


def _subset(items, step=41, n=96):
    """integrals spread over all 32 functions: 2D (PROP1) and 3D (PROP3) loops, many tables"""
    return [items[(i * step) % len(items)] for i in range(n)]


@pytest.fixture(scope="module")
def dctx(gblib, w):
    c = Context(0)
    c.serve_start_device(ring_slots=16, max_items=2048, max_units=1 << 20, idle_seconds=0.05)
    ts, tl = _tables(c, w)
    yield c, ts, tl
    c.serve_stop()
    c.close()


def test_device_loop_equals_gb_get_and_oracle(dctx, w, oracle):
    c, _, tl = dctx
    k = 0.7
    items = serving.rhs_items(w, k)
    sub = _subset(items)
    got = c.submit(sub, tl, "fp64").wait(timeout=300)
    ref = np.array([c.get(g, tl, "fp64") for g in sub])
    assert _close(got, ref), np.max(np.abs(got - ref) / np.abs(ref))
    pairs = [(i, j) for i in range(0, 32, 7) for j in (0, 64, 127)]
    want = serving.oracle_subset(oracle, w, w["y0"], k, pairs)
    got2 = c.submit([items[i * 128 + j] for i, j in pairs], tl, "fp64").wait(timeout=300)
    assert np.max(np.abs(got2 - want) / np.abs(want)) <= 1e-12


def test_every_family_and_integrand_through_the_loop(dctx):
    """POLY on several families (one request mixes them) and the table integrands of the
    benchmark workloads: each equals gb_get FP64 to rounding."""
    from diffrg_gb300 import workloads as W
    from kat import random_args

    c, _, _ = dctx
    rng = np.random.default_rng(4)
    polys = [integral("4D", "POLY", n=(24, 8, 6, 6), k=0.7, x_extent=1.5, args=random_args(rng)),
             integral("ANGLE_FTQ0", "POLY", n=(32, 10), k=0.6, T=0.2, x_extent=1.2,
                      args=random_args(rng, q0_rational=(0.2, 1.1))),
             integral("CART3", "POLY", n=(12, 10, 8), k=1.0, args=random_args(rng)),
             integral("1D", "POLY", n=(64,), k=0.9, x_extent=2.0, args=random_args(rng))]
    got = c.submit(polys, (), "fp64").wait(timeout=120)
    assert _close(got, [c.get(g, (), "fp64") for g in polys])
    for make, idx in ((W.c1, range(0, 64, 16)), (W.c2, range(0, 384, 97)), (W.c5, range(0, 128, 63))):
        wl = make()
        items, tabs = W.engine_items(wl)
        T = [c.table(s, d) for s, d in tabs]
        sub = [items[i] for i in idx]
        got = c.submit(sub, T, "fp64").wait(timeout=300)
        assert _close(got, [c.get(g, T, "fp64") for g in sub]), wl["name"]
        for t in T:
            t.close()


def test_alone_equals_in_mix_from_several_threads(dctx, w):
    c, _, tl = dctx
    items = serving.rhs_items(w, 0.55)
    probe = _subset(items, step=53, n=64)
    alone = c.submit(probe, tl, "fp64").wait(timeout=300)
    results, errors = {}, []

    def worker(tid):
        try:
            rng = np.random.default_rng(tid)
            for rep in range(4):
                lo = int(rng.integers(0, len(items) - 48))
                t_other = c.submit(items[lo:lo + 48], tl, "fp64")
                t_probe = c.submit(probe, tl, "fp64")
                t_other.wait(timeout=300)
                results[(tid, rep)] = t_probe.wait(timeout=300)
        except Exception as e:  # noqa: BLE001 -- reported below
            errors.append(repr(e))

    ths = [threading.Thread(target=worker, args=(i,)) for i in range(4)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    assert not errors, errors
    assert len(results) == 16
    for v in results.values():
        assert np.array_equal(v, alone)
    st = c.stats()
    assert st["completed"] >= 33 and 0 < st["p50_latency_s"] <= st["p99_latency_s"] <= st["max_latency_s"]


def test_latency_is_stamped_at_completion(dctx, w):
    """The watcher thread stamps a request's completion when its done flag rises, not when the
    caller gets round to waiting for it."""
    c, _, tl = dctx
    items = _subset(serving.rhs_items(w, 0.75), step=31, n=16)
    c.submit(items, tl, "fp64").wait(timeout=120)  # warm: axes, module
    c.reset_stats()
    t = c.submit(items, tl, "fp64")
    time.sleep(0.5)
    t.wait(timeout=120)
    st = c.stats()
    assert st["completed"] == 1 and st["max_latency_s"] < 0.25, st


def test_small_request_overtakes_a_large_one(dctx, w):
    """A request of at most 2^22 grid points goes to the express lane: submitted right behind a
    large request (1024 3D integrals), it finishes while the large one is still running, and
    both are exact."""
    c, _, tl = dctx
    items = serving.rhs_items(w, 0.9)
    per = len(w["p"])
    big = [items[i * per + j] for i in range(1, serving.N_FUNC, 2) for j in range(per)][:1024]
    probe = items[:8]  # 2D integrals
    c.submit(probe, tl, "fp64").wait(timeout=120)  # warm
    c.submit(big[:8], tl, "fp64").wait(timeout=120)
    tb = c.submit(big, tl, "fp64")
    tp = c.submit(probe, tl, "fp64")
    got_p = tp.wait(timeout=300)
    assert tb.poll() is None  # the large request is still running
    got_b = tb.wait(timeout=300)
    assert _close(got_p, [c.get(g, tl, "fp64") for g in probe])
    sub = big[::97]
    assert _close(got_b[::97], [c.get(g, tl, "fp64") for g in sub])


def test_request_reads_one_table_epoch(dctx, w):
    c, ts, tl = dctx
    items = _subset(serving.rhs_items(w, 0.8), step=29, n=128)
    yA, yB = w["y0"], np.clip(w["y0"] * 1.07, 0.5, 1.5)
    c.update_tables([(ts[i], yA[i]) for i in range(serving.N_FUNC)])
    refA = c.submit(items, tl, "fp64").wait(timeout=300)
    assert _close(refA, [c.get(g, tl, "fp64") for g in items])
    c.update_tables([(ts[i], yB[i]) for i in range(serving.N_FUNC)])
    refB = c.submit(items, tl, "fp64").wait(timeout=300)
    assert _close(refB, [c.get(g, tl, "fp64") for g in items])
    assert not _close(refA, refB, 1e-6)
    for rep in range(3):
        c.update_tables([(ts[i], yA[i]) for i in range(serving.N_FUNC)])
        t1 = c.submit(items, tl, "fp64")
        c.update_tables([(ts[i], yB[i]) for i in range(serving.N_FUNC)])  # waits for t1
        t2 = c.submit(items, tl, "fp64")
        assert np.array_equal(t1.wait(timeout=300), refA), rep
        assert np.array_equal(t2.wait(timeout=300), refB), rep
    c.update_tables([(ts[i], w["y0"][i]) for i in range(serving.N_FUNC)])


def test_admission_by_ring_capacity(gblib, w):
    c = Context(0)
    try:
        c.serve_start_device(ring_slots=2, max_items=64, max_units=4096, idle_seconds=0.02)
        _, tl = _tables(c, w)
        items = serving.rhs_items(w, 0.6)
        with pytest.raises(GbError) as e:  # more integrals than a slot holds
            c.submit(items[:65], tl, "fp64")
        assert e.value.code == capi.GB_EBUDGET
        big = integral("4D", "POLY", n=(128, 64, 32, 32), k=1.0, args=(0, 1))  # 8192 units > 4096
        with pytest.raises(GbError) as e:
            c.submit([big], (), "fp64")
        assert e.value.code == capi.GB_EBUDGET
        # ten requests through two slots, submitted back to back: each waits for its slot
        subs = [items[i * 16:i * 16 + 16] for i in range(10)]
        tks = [c.submit(s, tl, "fp64") for s in subs]
        for s, t in zip(subs, tks):
            assert _close(t.wait(timeout=300), [c.get(g, tl, "fp64") for g in s])
        st = c.stats()
        assert st["rejected"] == 2 and st["completed"] == 10
    finally:
        c.close()


def test_loop_runs_dry_then_relaunches(gblib, w):
    """With a 2 ms idle budget the loop ends by itself once the work is done: every CTA records
    an idle exit and the kernel is gone; the next submit launches it again and its results are
    exact.  No fault and no hang: the idle wait is a bounded clock64 spin."""
    c = Context(0)
    try:
        c.serve_start_device(ring_slots=4, max_items=256, max_units=1 << 16, idle_seconds=0.002)
        _, tl = _tables(c, w)
        items = _subset(serving.rhs_items(w, 0.65), step=37, n=32)
        ref = c.submit(items, tl, "fp64").wait(timeout=120)
        assert _close(ref, [c.get(g, tl, "fp64") for g in items])
        time.sleep(0.2)
        info = c.device_loop_info()
        assert not info["running"]
        assert info["launches"] >= 1
        import ctypes as C

        dev, nsm = C.c_int(), C.c_int()
        capi.lib().gb_device_info(c.h, C.byref(dev), C.byref(nsm))
        assert info["idle_exits"] >= nsm.value * info["launches"]
        launches = info["launches"]
        assert np.array_equal(c.submit(items, tl, "fp64").wait(timeout=120), ref)
        assert c.device_loop_info()["launches"] == launches + 1
    finally:
        c.close()
