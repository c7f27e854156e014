"""GPU: the continuously batching request loop (gb_serve_* / gb_submit / gb_wait).

* served results equal the same integrals run as one gb_batch, bit for bit, and the FP64
  oracle within 1e-9 (FP32-compensated) / 1e-12 (FP64);
* a request gives bit-identical results alone and in a mix of concurrent requests;
* a request in flight reads one table epoch, never a mixture (table updates are ordered);
* cancel / poll / unknown tickets / HBM-budget admission;
* the node pool evicts unheld axes, so an RG flow with a new k per stage never runs out;
* one Cash-Karp step of the C4 flow, FP32-compensated against FP64;
* a small request behind a large one finishes first (one CTA per unit, priority streams).
"""

import numpy as np
import pytest

from diffrg_gb300 import capi, serving
from diffrg_gb300.capi import GbError
from diffrg_gb300.engine import Context, integral

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def w():
    return serving.c4()


@pytest.fixture(scope="module")
def sctx(gblib):
    c = Context(0)
    c.serve_start(8, 2048)
    yield c
    c.serve_stop()
    c.close()


@pytest.fixture(scope="module")
def tabs(sctx, w):
    ts = [sctx.table(w["spec"], w["y0"][i]) for i in range(serving.N_FUNC)]
    return ts, [ts[i] for i in serving.table_order()]


def serve_all(ctx, items, tlist, sizes, precision="fp32c"):
    tk = []
    off = 0
    for s in sizes:
        tk.append((off, ctx.submit(items[off:off + s], tlist, precision)))
        off += s
    out = np.empty(len(items))
    for o, t in tk:
        out[o:o + t.n] = t.wait(timeout=300)
    return out


def test_small_request_is_not_held_behind_a_large_one(sctx, tabs, w):
    """Serving grids run one CTA per work unit, each retiring after its unit, and small batches
    go to high-priority streams: a small request submitted right behind a large one (2048 3D
    integrals, the largest C4 request) finishes while the large one is still running, with the
    same bits as alone."""
    _, tlist = tabs
    items = serving.rhs_items(w, 0.85)
    per = len(w["p"])
    big = [items[i * per + j] for i in range(1, serving.N_FUNC, 2) for j in range(per)][:2048]
    probe = items[:8]
    alone = sctx.submit(probe, tlist, "fp32c").wait(timeout=120)
    sctx.submit(big, tlist, "fp32c").wait(timeout=120)  # warm: arenas, axes
    overtaken = 0
    for _ in range(3):
        tb = sctx.submit(big, tlist, "fp32c")
        got = sctx.submit(probe, tlist, "fp32c").wait(timeout=120)
        overtaken += tb.poll() is None
        tb.wait(timeout=300)
        assert np.array_equal(got, alone)
    assert overtaken >= 2


def test_served_equals_batch_and_oracle(sctx, tabs, w, oracle):
    _, tlist = tabs
    k = 0.7
    items = serving.rhs_items(w, k)
    sizes = serving.request_sizes(np.random.default_rng(3), len(items), 8, 2048)
    served = serve_all(sctx, items, tlist, sizes)
    b = sctx.batch(items, tlist, "fp32c")
    ref = b.get()
    b.close()
    assert np.array_equal(served, ref)
    pairs = [(i, j) for i in range(0, 32, 5) for j in (0, 77, 127)]
    want = serving.oracle_subset(oracle, w, w["y0"], k, pairs)
    got = np.array([served[i * 128 + j] for i, j in pairs])
    err = np.abs(got - want) / np.abs(want)
    assert np.max(err) <= 1e-9, err


def test_served_values_match_golden(sctx, tabs, w):
    import json
    import os

    _, tlist = tabs
    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "workloads_oracle.json")))
    rec = gold["workloads"]["C4"]
    items = serving.rhs_items(w, rec["k"])
    sub = [items[i * 128 + j] for i, j in rec["pairs"]]
    want = np.array([float(v) for v in rec["values"]])
    for prec, tol in (("fp64", 1e-12), ("fp32c", 1e-9)):
        got = sctx.submit(sub, tlist, prec).wait(timeout=300)
        assert np.max(np.abs(got - want) / np.abs(want)) <= tol, prec


def test_fp64_requests_match_oracle(sctx, tabs, w, oracle):
    _, tlist = tabs
    k = 0.9
    items = serving.rhs_items(w, k)
    pairs = [(0, 5), (1, 60), (6, 127), (11, 0)]
    sub = [items[i * 128 + j] for i, j in pairs]
    got = sctx.submit(sub, tlist, "fp64").wait(timeout=300)
    want = serving.oracle_subset(oracle, w, w["y0"], k, pairs)
    assert np.max(np.abs(got - want) / np.abs(want)) <= 1e-12


def test_alone_equals_in_mix_bitwise(sctx, tabs, w):
    _, tlist = tabs
    items = serving.rhs_items(w, 0.55)
    probe = items[1000:1100]  # crosses function boundaries: 2D and 3D integrals, many tables
    alone = sctx.submit(probe, tlist).wait(timeout=300)
    sctx.reset_stats()
    rng = np.random.default_rng(11)
    for rep in range(3):
        tk = []
        order = rng.permutation(6)
        for m in order:
            lo = int(m) * 600
            tk.append(sctx.submit(items[lo:lo + 600], tlist))
            if m == 2:
                tk.append(("probe", sctx.submit(probe, tlist)))
        mixed = None
        for t in tk:
            if isinstance(t, tuple):
                mixed = t[1].wait(timeout=300)
            else:
                t.wait(timeout=300)
        assert np.array_equal(mixed, alone), rep
    st = sctx.stats()
    assert st["completed"] == 21 and st["batches_launched"] >= 2
    assert 0 < st["p50_latency_s"] <= st["p99_latency_s"] <= st["max_latency_s"]


def test_request_reads_one_table_epoch(sctx, tabs, w):
    ts, tlist = tabs
    items = serving.rhs_items(w, 0.8)[1024:3072]
    yA = w["y0"]
    yB = np.clip(w["y0"] * 1.07, 0.5, 1.5)
    for i in range(serving.N_FUNC):
        ts[i].update(yA[i])
    bA = sctx.batch(items, tlist).get()
    for i in range(serving.N_FUNC):
        ts[i].update(yB[i])
    bB = sctx.batch(items, tlist).get()
    assert not np.array_equal(bA, bB)
    for rep in range(3):
        sctx.update_tables([(ts[i], yA[i]) for i in range(serving.N_FUNC)])
        t1 = sctx.submit(items, tlist)
        # one group of updates, issued while t1 is queued or running
        sctx.update_tables([(ts[i], yB[i]) for i in range(serving.N_FUNC)])
        t2 = sctx.submit(items, tlist)
        r1 = t1.wait(timeout=300)
        r2 = t2.wait(timeout=300)
        assert np.array_equal(r1, bA) or np.array_equal(r1, bB), rep
        assert np.array_equal(r2, bB), rep
    for i in range(serving.N_FUNC):
        ts[i].update(w["y0"][i])


def test_poll_cancel_and_tickets(gblib, w):
    c = Context(0)
    try:
        c.serve_start(1, 2048)
        ts = [c.table(w["spec"], w["y0"][i]) for i in range(serving.N_FUNC)]
        tlist = [ts[i] for i in serving.table_order()]
        items = serving.rhs_items(w, 0.6)
        big = c.submit(items[128:2176], tlist, "fp32c")  # ~0.5e9 points on the one slot
        small = c.submit(items[:8], tlist, "fp64")  # another precision: its own batch
        canceled = small.cancel()
        r = big.poll()
        assert r is None or r.shape == (2048,)
        big_res = big.wait(timeout=300) if r is None else r
        assert np.all(np.isfinite(big_res))
        if canceled:
            with pytest.raises(GbError) as e:
                small.wait(timeout=60)
            assert e.value.code == capi.GB_ECANCELED
        else:
            assert np.all(np.isfinite(small.wait(timeout=60)))
        with pytest.raises(GbError) as e:  # a consumed ticket is unknown
            big.wait(timeout=1)
        assert e.value.code == capi.GB_EINVAL
        # a finished request stays pollable until consumed
        t = c.submit(items[:8], tlist)
        res = t.wait(timeout=60)
        assert res.shape == (8,)
    finally:
        c.close()


def test_hbm_budget_admission(gblib, w):
    c = Context(0, budget_bytes=1 << 20)
    try:
        c.serve_start(2, 8192)
        ts = [c.table(w["spec"], w["y0"][i]) for i in range(serving.N_FUNC)]
        tlist = [ts[i] for i in serving.table_order()]
        items = serving.rhs_items(w, 0.6)
        with pytest.raises(GbError) as e:  # descriptors alone exceed the budget
            c.submit(items, tlist)
        assert e.value.code == capi.GB_EBUDGET
        # fits at submit, but its work units (3D integrals) do not fit the budget at launch
        t = c.submit(items[:2048], tlist)
        with pytest.raises(GbError) as e:
            t.wait(timeout=120)
        assert e.value.code == capi.GB_EBUDGET
        ok = c.submit(items[:16], tlist).wait(timeout=60)
        assert np.all(np.isfinite(ok))
        st = c.stats()
        assert st["rejected"] >= 2 and st["bytes_in_use"] <= st["bytes_budget"]
    finally:
        c.close()


def test_node_pool_evicts_unheld_axes(ctx, oracle):
    """600 RG scales x a 4096-node radial axis exceed the 2^21-node pool: unheld axes are
    evicted and reused; a batch built before the churn keeps its axes and its result."""
    from diffrg_gb300.workloads import poly_args

    args = poly_args(q=(1.0, 0.5, 0, 0, 0, 0))
    g0 = integral("1D", "POLY", d=3, n=(4096,), k=0.5, x_extent=2.0, args=args)
    keep = ctx.batch([g0], precision="fp64")
    v0 = keep.get()[0]
    for m in range(600):
        k = 0.5 + 1e-3 * (m + 1)
        b = ctx.batch([integral("1D", "POLY", d=3, n=(4096,), k=k, x_extent=2.0, args=args)], precision="fp64")
        v = b.get()[0]
        b.close()
        if m % 150 == 0:
            d = oracle.family_desc("1D", d=3, n=(4096,), x_extent=2.0)
            want = oracle.family(d, "POLY", k, args[None, :])[0]
            assert abs(v - want) <= 1e-12 * abs(want)
    assert keep.get()[0] == v0
    keep.close()


def test_c4_flow_step_fp32c_vs_fp64(gblib, w):
    c = Context(0)
    try:
        c.serve_start(8, 2048)
        out = {}
        for prec in ("fp32c", "fp64"):
            f = serving.Flow(c, w, precision=prec, rate=None)
            y, err = serving.cash_karp_step(f.rhs, 0.0, w["y0"].copy(), 0.2)
            out[prec] = y
            assert f.rhs_evals == 6 and f.integrals == 6 * 4096
            f.close()
        y32, y64 = out["fp32c"], out["fp64"]
        assert np.all(np.isfinite(y32)) and 0.4 < y32.min() and y32.max() < 1.6
        # stage values enter the tables rounded to FP32, so a 1e-10 difference between the two
        # runs can flip one table entry by an FP32 ulp (6e-8) at a later stage
        assert np.max(np.abs(y32 - y64) / np.abs(y64)) <= 1e-8
        st = c.stats()
        assert st["completed"] >= 2 * 6 * 2 and st["rejected"] == 0
    finally:
        c.close()


def test_event_log_lines_are_json(gblib, tmp_path):
    """GBINT_LOG=<file>: batch creation, serving launches/completions and autotuning are logged
    as one JSON object per line."""
    import json
    import os
    import subprocess
    import sys

    log = tmp_path / "gbint.jsonl"
    code = r'''
import numpy as np
from diffrg_gb300 import serving
from diffrg_gb300.engine import Context
w = serving.c4()
ctx = Context(0)
ts = [ctx.table(w["spec"], w["y0"][i]) for i in range(serving.N_FUNC)]
tl = [ts[i] for i in serving.table_order()]
items = serving.rhs_items(w, 0.5)
b = ctx.batch(items[:64], tl); b.get(); b.close()
ctx.serve_start(2, 512)
tk = [ctx.submit(items[i * 100:(i + 1) * 100], tl) for i in range(5)]
for t in tk: t.wait(timeout=120)
ctx.autotune(items[:256], tl)
ctx.close()
'''
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, GBINT_LOG=str(log), PYTHONPATH=root)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    events = [json.loads(l) for l in log.read_text().splitlines()]
    kinds = {e["event"] for e in events}
    assert {"batch_create", "serve_launch", "serve_done", "autotune"} <= kinds
    done = [e for e in events if e["event"] == "serve_done"]
    assert sum(e["integrals"] for e in done) == 500 and all(e["ok"] == 1 for e in done)
    assert all(e["t"] >= 0 for e in events)


def test_concurrent_host_threads(gblib, w):
    """Many host threads using one context at once (gets, batches, submits, table updates):
    every result equals the serial one bit for bit."""
    import threading

    c = Context(0)
    try:
        c.serve_start(4, 1024)
        ts = [c.table(w["spec"], w["y0"][i]) for i in range(serving.N_FUNC)]
        tl = [ts[i] for i in serving.table_order()]
        items = serving.rhs_items(w, 0.65)
        picks = list(range(0, 4096, 97))
        b = c.batch([items[i] for i in picks], tl, "fp32c")
        ref = b.get()
        b.close()
        errors = []

        def worker(tid):
            try:
                for rep in range(4):
                    if (tid + rep) % 3 == 0:
                        got = c.submit([items[i] for i in picks], tl).wait(timeout=300)
                    elif (tid + rep) % 3 == 1:
                        bb = c.batch([items[i] for i in picks], tl, "fp32c")
                        got = bb.get()
                        bb.close()
                    else:
                        got = np.array([c.batch([items[i]], tl, "fp32c").get()[0] for i in picks[:5]])
                        if not np.array_equal(got, ref[:5]):
                            errors.append((tid, rep, "single"))
                        continue
                    if not np.array_equal(got, ref):
                        errors.append((tid, rep))
            except Exception as e:  # surfaced below
                errors.append((tid, repr(e)))

        th = [threading.Thread(target=worker, args=(t,)) for t in range(8)]
        for t in th:
            t.start()
        for t in th:
            t.join(timeout=600)
        assert not errors, errors[:5]
    finally:
        c.close()


def test_served_finite_t_and_vertex_requests(sctx):
    """Requests of the finite-T loop (C2: mode-interpolated slices) and the 4D vertex (C5:
    cos-axis slices) through the request loop, interleaved, in small requests: bit-identical to
    one batch of the same integrals."""
    from diffrg_gb300 import workloads as W
    import test_gpu_parity as TP

    w2, w5 = TP.subset(W, "C2"), TP.subset(W, "C5")
    i2, t2 = W.engine_items(w2)
    i5, t5 = W.engine_items(w5)
    for g in i5:
        g.table_base = 1
    T = [sctx.table(s, d) for s, d in t2 + t5]
    items = i2[:6] + i5 + i2[6:]
    sizes = [3, 3, 2, 4, 5, 7, 6]
    served = serve_all(sctx, items, T, sizes)
    b = sctx.batch(items, T, "fp32c")
    ref = b.get()
    b.close()
    for t in T:
        t.close()
    assert np.array_equal(served, ref)
