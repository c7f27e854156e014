"""GPU parity: every path of libgbint against the FP64 CPU oracle, through the C ABI.

Tolerances (relative, per integral):
  * FP64 fused kernels and the reference-pattern FP64 path vs oracle: 1e-12 (same quadrature,
    different summation order);
  * FP32-compensated kernels vs oracle: TOL32 below, measured on GB300 and fixed here;
  * polynomial known answers vs closed forms: the reference's own tolerances (kat.py).
"""
import math

import numpy as np
import pytest

from kat import CASES, analytic, random_args

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
# FP32-compensated (default, double-float per-point form) vs FP64 oracle: the 1e-9 target,
# max over the integrals of the test subset
TOL32 = {"C1": 1e-9, "C2": 1e-9, "C3": 1e-9, "C5": 1e-9}
# fast FP32 form (explicit opt-in): ~5e-8 rms per point, residual bias ~1e-9
TOL32F = 2e-8


@pytest.fixture(scope="module")
def W():
    from diffrg_gb300 import workloads

    return workloads


def rel(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


# ------------------------------------------------------------------ QuadratureProvider
@pytest.mark.parametrize("n", [1, 2, 5, 16, 64, 128, 256, 1000])
def test_gl_provider_matches_oracle(ctx, oracle, n):
    x, w = ctx.gl(n)
    xo, wo = oracle.gauss_legendre(n)
    assert np.max(np.abs(x - xo)) <= 2e-16
    assert np.max(np.abs(w - wo)) <= 4e-16 * max(1, n / 64)


def _device_array(ptr, n, typestr):
    import torch

    class _View:
        pass

    v = _View()
    # torch takes no read-only flag (it must be False); the view is only copied to the host
    v.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "strides": None,
                                  "version": 3}
    return torch.as_tensor(v, device="cuda").cpu().numpy()


@pytest.mark.parametrize("qtype", [0, 1, 2, 3, 4])
def test_rule_types_host_and_device(ctx, qtype):
    """QuadratureProvider::get_points/get_device_points with a QuadratureType: the context's
    cached rule equals the host-only rule, and its FP64 / FP32 device copies hold the same values."""
    from diffrg_gb300 import engine as E

    n = 24
    x, w = ctx.rule(qtype, n)
    xh, wh = E.quad_rule_host(qtype, n)
    assert np.array_equal(x, xh) and np.array_equal(w, wh)
    for dtype, typestr, npt in ((0, "<f8", np.float64), (1, "<f4", np.float32)):
        dx, dw = ctx.rule_device(qtype, n, dtype)
        assert np.array_equal(_device_array(dx, n, typestr), x.astype(npt))
        assert np.array_equal(_device_array(dw, n, typestr), w.astype(npt))


@pytest.mark.parametrize("T,E", [(0.05, 1.0), (0.2, 1.0), (1.0, 1.0), (0.1, 0.3), (0.001, 1.0), (0.0, 2.0)])
def test_matsubara_provider_matches_oracle(ctx, oracle, T, E):
    x, w, tr = ctx.matsubara(T, E)
    xo, wo, tro = oracle.matsubara(T, E, step=2, min_size=32, max_size=128, vacuum=48, precision_factor=0)
    assert tr == tro and x.size == xo.size
    assert np.max(rel(x, xo)) < 1e-13
    assert np.max(rel(w, wo)) < 1e-12


def test_matsubara_provider_closed_form(ctx):
    for T in (0.03, 0.3, 0.9):
        x, w, tr = ctx.matsubara(T, 1.0)
        s = tr * 1.0 + np.sum(w * 2.0 / (1.0 + x * x))
        assert abs(s - 0.5 / math.tanh(0.5 / T)) < 1e-13 * s


# ------------------------------------------------------------------ families, polynomial KERNEL
def engine_poly(fam, seed):
    from diffrg_gb300.engine import integral

    rng = np.random.default_rng(seed)
    kw = dict(CASES[fam])
    n = kw.pop("n")
    d = kw.pop("d")
    k = rng.uniform(0.3, 1.0)
    xe = rng.uniform(1.0, 2.0)
    T = kw.get("T", 0.0)
    args = random_args(rng, q0_rational=(T, rng.uniform(0.8, 1.2))) if fam.endswith("FTQ0") else random_args(rng)
    if fam.endswith("FTX0"):
        kw["x0_extent"] = kw["x0_summands"] * 10 * 2 * math.pi * T / k * 1.5 + 1000.0 / k
    g = integral(fam, "POLY", n=n, k=k, d=d, x_extent=xe, x0_extent=kw.get("x0_extent", 0.0),
                 x0_summands=kw.get("x0_summands", 0), T=T, qmin=kw.get("qmin", (-math.pi,) * 3),
                 qmax=kw.get("qmax", (math.pi,) * 3), args=args)
    return g, n, d, k, xe, args, kw


@pytest.mark.parametrize("fam", list(CASES))
def test_family_poly_fp64(ctx, oracle, fam):
    from test_oracle_families import oracle_family

    for seed in (11, 12):
        g, n, d, k, xe, args, kw = engine_poly(fam, seed)
        got = ctx.get(g, (), "fp64")
        ref = oracle_family(oracle, fam, n, d, k, xe, args, kw)
        assert abs(got - ref) <= TOL64 * max(abs(ref), 1e-3), (fam, got, ref)
        ana = analytic(fam, args, k, d=d, x_extent=xe, **kw)
        tol = 5e-5 if fam.endswith("FTQ0") else 1e-4
        assert abs(got - ana) <= tol * max(1.0, abs(ana))


def test_family_batch_matches_single_gets(ctx):
    gs = [engine_poly(f, 5)[0] for f in ("ANGLE", "4D", "3DPX0", "FTX0", "4D_FTQ0", "CART3")]
    b = ctx.batch(gs, (), "fp64")
    many = b.get()
    b.close()
    one = np.array([ctx.get(g, (), "fp64") for g in gs])
    assert np.array_equal(many, one)


# ------------------------------------------------------------------ benchmark workloads
def subset(W, name):
    w = getattr(W, name.lower())()
    if name == "C2":
        sel = np.concatenate([np.arange(0, 128, 16), 128 + np.arange(0, 128, 16), 256 + np.arange(0, 128, 16)])
        w["p"], w["T"] = w["p"][sel], w["T"][sel]
    elif name == "C3":
        rng = np.random.default_rng(3)
        sel = rng.choice(4096, 48, replace=False)
        w["orders"], w["P"] = w["orders"][sel], w["P"][sel]
    elif name == "C5":
        sel = np.array([0, 21, 63, 64, 100, 127])
        w["P"], w["alpha"] = w["P"][sel], w["alpha"][sel]
    return w


def run_engine(ctx, W, w, prec):
    items, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    b = ctx.batch(items, T, prec)
    out = b.get()
    b.close()
    for t in T:
        t.close()
    return out


@pytest.mark.parametrize("name", ["C1", "C2", "C3", "C5"])
def test_workload_fp64_matches_oracle(ctx, oracle, W, name):
    w = subset(W, name)
    got = run_engine(ctx, W, w, "fp64")
    ref = W.oracle_values(w, oracle)
    assert np.max(rel(got, ref)) <= TOL64


@pytest.mark.parametrize("name", ["C1", "C2", "C3", "C5"])
def test_workload_fp32c_matches_oracle(ctx, oracle, W, name):
    w = subset(W, name)
    got = run_engine(ctx, W, w, "fp32c")
    ref = W.oracle_values(w, oracle)
    err = rel(got, ref)
    print("%s fp32c max rel err %.3e  median %.3e" % (name, err.max(), np.median(err)))
    assert np.all(np.isfinite(got))
    assert err.max() <= TOL32[name]


@pytest.mark.parametrize("name", ["C1", "C2", "C3", "C5"])
def test_whole_workload_fp32c_matches_oracle(ctx, oracle, W, name):
    """Every integral of each benchmark workload (C3: all 4096 uneven 3D loops; C5: all 128
    4.19M-point vertex loops), FP32-compensated, against the FP64 oracle on all host cores."""
    import os

    w = getattr(W, name.lower())()
    got = run_engine(ctx, W, w, "fp32c")
    ref = W.oracle_values(w, oracle, threads=os.cpu_count() or 1)
    err = rel(got, ref)
    print("%s all %d integrals: fp32c max rel err %.3e median %.3e" % (name, len(got), err.max(), np.median(err)))
    assert np.all(np.isfinite(got))
    assert err.max() <= TOL32[name]


@pytest.mark.parametrize("name", ["C1", "C2", "C3", "C5"])
def test_workload_fp32_fast_matches_oracle(ctx, oracle, W, name):
    w = subset(W, name)
    got = run_engine(ctx, W, w, "fp32f")
    ref = W.oracle_values(w, oracle)
    err = rel(got, ref)
    print("%s fp32f max rel err %.3e  median %.3e" % (name, err.max(), np.median(err)))
    assert err.max() <= TOL32F


@pytest.mark.parametrize("name", ["C1", "C2", "C3", "C5"])
def test_workloads_match_golden_values(ctx, W, name):
    """Engine (FP64 and FP32C) against the committed oracle values of fixed subsets."""
    import json
    import os

    gold = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "workloads_oracle.json")))
    rec = gold["workloads"][name]
    sub = np.array(rec["subset"])
    want = np.array([float(v) for v in rec["values"]])
    w = getattr(W, name.lower())()
    if name == "C2":
        w["p"], w["T"] = w["p"][sub], w["T"][sub]
    elif name == "C3":
        w["orders"], w["P"] = w["orders"][sub], w["P"][sub]
    elif name == "C5":
        w["P"], w["alpha"] = w["P"][sub], w["alpha"][sub]
    else:
        w["p"] = w["p"][sub]
    assert np.max(rel(run_engine(ctx, W, w, "fp64"), want)) <= TOL64
    assert np.max(rel(run_engine(ctx, W, w, "fp32c"), want)) <= TOL32[name]


@pytest.mark.parametrize("name", ["C1", "C5"])
def test_reference_pattern_matches_oracle(ctx, oracle, W, name):
    w = subset(W, name)
    items, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    b = ctx.batch(items, T, "fp64")
    got = b.run_plain(8)
    b.close()
    ref = W.oracle_values(w, oracle)
    assert np.max(rel(got, ref)) <= TOL64


def c2_items_with_omega(W, w, Om):
    from diffrg_gb300.engine import integral

    return [integral("QLOOP_T", "FTLOOP", n=(w["nq"], w["nc"]), k=1.0, x_extent=w["qmax"], x0_summands=w["M"],
                     T=T, args=(0.0, p, T, Om)) for p, T in zip(w["p"], w["T"])]


@pytest.mark.parametrize("prec", ["fp32c", "fp32f", "fp64"])
def test_c2_twin_signs_are_bitwise_the_two_sign_sum(ctx, W, prec):
    """Omega = 0: the +-w evaluations of the finite-T loop are one doubled evaluation; a
    negligible Omega (1e-300, which leaves every w +- Omega unchanged) takes the two-sign path
    and must give the same bits."""
    w = subset(W, "C2")
    _, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    out = []
    for Om in (0.0, 1e-300):
        b = ctx.batch(c2_items_with_omega(W, w, Om), T, prec)
        out.append(b.get())
        b.close()
    for t in T:
        t.close()
    assert np.array_equal(out[0], out[1])


def test_c2_nonzero_external_frequency_matches_oracle(ctx, oracle, W):
    w = subset(W, "C2")
    _, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    Om = 2 * math.pi * 0.2 * 3  # a bosonic external frequency of the T = 0.2 rows
    b = ctx.batch(c2_items_with_omega(W, w, Om), T, "fp32c")
    got = b.get()
    b.close()
    b = ctx.batch(c2_items_with_omega(W, w, Om), T, "fp64")
    got64 = b.get()
    b.close()
    for t in T:
        t.close()
    ref = oracle.w2(w["tables"][0], w["M"], w["nq"], w["nc"], w["qmax"], w["p"], w["T"], Omega=Om)
    assert np.max(rel(got64, ref)) <= TOL64
    assert np.max(rel(got, ref)) <= TOL32["C2"]


# ------------------------------------------------------------------ batching semantics
def test_alone_and_in_mix_are_bitwise_identical(ctx, W):
    """Each integral's result is independent of what else is in the launch (deterministic
    per-integral finish), for the FP32-compensated and FP64 kernels."""
    w = subset(W, "C3")
    items, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    for prec in ("fp32c", "fp64"):
        b = ctx.batch(items, T, prec)
        mix = b.get()
        b.close()
        for i in (0, 7, 31):
            b1 = ctx.batch([items[i]], T, prec)
            alone = b1.get()[0]
            b1.close()
            assert alone == mix[i]
    for t in T:
        t.close()


def test_graph_replay_matches_direct_run(ctx, W):
    w = subset(W, "C2")
    items, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    b = ctx.batch(items, T, "fp32c")
    direct = b.get()
    for _ in range(3):
        b.run_graph()
        assert np.array_equal(b.results(), direct)
    b.close()
    for t in T:
        t.close()


def test_captured_sweep_replays_every_batch(ctx, W):
    """One graph holding the runs of three batches (C1, C3, C5 subsets) replays them all;
    each replay gives the direct runs' bits; table updates are refused while capturing and
    the replay reads tables as they are when it runs."""
    from diffrg_gb300.capi import GbError

    Ts, bs, direct = [], [], []
    for name in ("C1", "C3", "C5"):
        w = subset(W, name)
        items, tabs = W.engine_items(w)
        T = [ctx.table(s, d) for s, d in tabs]
        b = ctx.batch(items, T, "fp32c")
        direct.append(b.get())
        Ts.append((T, tabs))
        bs.append(b)
    bad = []

    def body():
        for b in bs:
            b.run()
        try:
            Ts[0][0][0].update(Ts[0][1][0][1])
        except GbError as e:
            bad.append(e.code)

    g = ctx.capture(body)
    assert bad == [1]
    assert g.kernel_launches >= 6
    for _ in range(3):
        g.replay()
        for b, d in zip(bs, direct):
            assert np.array_equal(b.results(), d)
    # the replay reads the current table contents
    T1, tabs1 = Ts[0]
    T1[0].update(tabs1[0][1] * np.float32(1.5))
    g.replay()
    changed = bs[0].results()
    assert not np.array_equal(changed, direct[0])
    bs[0].run()
    assert np.array_equal(bs[0].results(), changed)
    T1[0].update(tabs1[0][1])
    g.close()
    for b in bs:
        b.close()
    for T, _ in Ts:
        for t in T:
            t.close()


def test_autotuner_choices_cache_and_accuracy(ctx, oracle, W, tmp_path):
    """gb_autotune picks a built CTA width per kernel kind, writes the per-GPU cache, reuses it
    on the next call, and the tuned batches keep the accuracy bar."""
    cache = str(tmp_path / "tune.txt")
    try:
        for name, slot in (("C3", 7 + 8), ("C1", 1 + 8)):
            w = subset(W, name)
            items, tabs = W.engine_items(w)
            T = [ctx.table(s, d) for s, d in tabs]
            got = ctx.autotune(items, T, "fp32c", cache_path=cache)
            assert got.get(slot) in (128, 256, 512)
            rep = {k["slot"]: k for k in ctx.tune_report()["kinds"]}[slot]
            assert not rep["cached"] and rep["chosen_ms"] > 0 and rep["default_ms"] > 0
            assert rep["chosen_ms"] <= rep["default_ms"]
            want = {"threads", "rows_per_thread", "unit_order"} | ({"inner_split"} if name == "C3" else set())
            assert set(rep["steps"]) == want
            assert all(len(rep["steps"][k]) == (2 if k == "unit_order" else 3) for k in want)
            sched = ctx.tune_get_schedule(slot)
            assert sched == rep["chosen"]
            lines = open(cache).read().splitlines()
            assert any(l.split("|")[2] == str(slot) for l in lines)
            again = ctx.autotune(items, T, "fp32c", cache_path=cache)
            assert again[slot] == got[slot]
            assert ctx.tune_get_schedule(slot) == sched
            assert {k["slot"]: k for k in ctx.tune_report()["kinds"]}[slot]["cached"]
            b = ctx.batch(items, T, "fp32c")
            val = b.get()
            b.close()
            ref = W.oracle_values(w, oracle)
            assert np.max(rel(val, ref)) <= TOL32[name]
            for t in T:
                t.close()
        with pytest.raises(Exception):
            ctx.tune_set(3, 96)
        with pytest.raises(Exception):
            ctx.tune_set_schedule(3, rows_per_thread=3)
    finally:
        for k in range(16):
            ctx.tune_set_schedule(k)


@pytest.mark.parametrize("name,slot", [("C1", 1 + 8), ("C2", 2 + 8), ("C3", 7 + 8), ("C5", 6 + 8)])
def test_work_unit_schedules_keep_accuracy(ctx, oracle, W, name, slot):
    """Every schedule (CTA width x rows per thread x inner split) meets the accuracy bar and is
    deterministic; the cost order changes only which CTA runs a unit, so its results equal the
    item order's bit for bit."""
    w = subset(W, name)
    items, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    ref = W.oracle_values(w, oracle)

    def run():
        b = ctx.batch(items, T, "fp32c")
        v = b.get()
        b.close()
        return v

    splits = (1, 2, 4) if name in ("C3", "C5") else (1,)
    shapes = [(256, 1, 1), (128, 4, 1), (512, 2, 1)] + [(256, 2, s) for s in splits[1:]] + [(128, 1, 4)] * (len(splits) > 1)
    try:
        for th, rpt, sp in shapes:
            ctx.tune_set_schedule(slot, th, rpt, sp, "item")
            sc = ctx.tune_get_schedule(slot)
            assert (sc["threads"], sc["rows_per_thread"], sc["inner_split"]) == (th, rpt, sp)
            v_item = run()
            assert np.max(rel(v_item, ref)) <= TOL32[name], (th, rpt, sp)
            assert np.array_equal(run(), v_item)
            ctx.tune_set_schedule(slot, th, rpt, sp, "cost")
            assert np.array_equal(run(), v_item), (th, rpt, sp)
    finally:
        ctx.tune_set_schedule(slot)
        for t in T:
            t.close()


def test_bounded_wait_times_out_and_context_survives(ctx, W):
    """A device-side wait that nothing completes gives up after its cycle limit, reports
    GB_ETIMEDOUT through the error word, and the context keeps computing correct results."""
    from diffrg_gb300 import capi

    w = subset(W, "C1")
    before = run_engine(ctx, W, w, "fp32c")
    for cycles in (1 << 10, 1 << 20):
        assert ctx.selftest_wait(cycles) == capi.GB_ETIMEDOUT
        assert "gave up" in ctx.last_error()
    assert ctx.selftest_wait(0) == capi.GB_EINVAL
    after = run_engine(ctx, W, w, "fp32c")
    assert np.array_equal(before, after)


def test_table_update_is_seen_by_next_run(ctx, oracle, W):
    w = subset(W, "C1")
    items, tabs = W.engine_items(w)
    spec, Z = tabs[0]
    t = ctx.table(spec, Z)
    b = ctx.batch(items, [t], "fp32c")
    first = b.get()
    Z2 = (Z * 1.1).astype(np.float32)
    t.update(Z2)
    assert t.epoch == 2
    second = b.get()
    w2 = dict(w)
    w2["tables"] = [(spec, Z2)]
    ref = W.oracle_values(w2, oracle)
    assert np.max(rel(second, ref)) <= TOL32["C1"]
    assert np.max(rel(first, second)) > 1e-3
    b.close()
    t.close()


@pytest.mark.parametrize("many", [False, True])
def test_table_update_rebuilds_cell_records(ctx, oracle, W, many):
    """C3's kernel reads its three point-dependent tables through per-cell records rebuilt on
    every update (single updates and gb_table_update_many): after an update the next run
    matches the oracle on the new data."""
    w = subset(W, "C3")
    items, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    b = ctx.batch(items, T, "fp32c")
    first = b.get()
    new = [(d * (1.0 + 0.05 * (k + 1))).astype(np.float32) for k, (_, d) in enumerate(tabs)]
    if many:
        ctx.update_tables([(t, d) for t, d in zip(T, new)])
    else:
        for t, d in zip(T, new):
            t.update(d)
    second = b.get()
    w2 = dict(w)
    w2["tables"] = [(s, d) for (s, _), d in zip(tabs, new)]
    ref = W.oracle_values(w2, oracle)
    assert np.max(rel(second, ref)) <= TOL32["C3"]
    assert np.max(rel(first, second)) > 1e-3
    b.close()
    for t in T:
        t.close()


def test_untrusted_propagator_series_cells(ctx, oracle, W):
    """C3's kernel reads B's propagator 1 / (Z(x) x + R(x)) from a per-cell series in t = x / c_j - 1;
    where the series is not trusted over a cell (a table whose value jumps 60 % from cell to cell
    puts the series' radius next to the cell), the kernel evaluates the cell from the value record
    and the regulator instead.  A B table alternating between 0.4 and 1.0 (most cells untrusted)
    and one with a single such jump both match the oracle."""
    w = subset(W, "C3")
    spec, zb = w["tables"][1]
    alt = np.where(np.arange(zb.size) % 2 == 0, 0.4, 1.0).astype(np.float32)
    jump = zb.copy()
    jump[120:] *= 0.4
    for zb2 in (alt, jump):
        w2 = dict(w)
        w2["tables"] = list(w["tables"])
        w2["tables"][1] = (spec, zb2)
        got = run_engine(ctx, W, w2, "fp32c")
        ref = W.oracle_values(w2, oracle)
        assert np.all(np.isfinite(got))
        assert np.max(rel(got, ref)) <= TOL32["C3"]


def test_errors_are_status_codes(ctx, W):
    from diffrg_gb300 import GbError
    from diffrg_gb300.engine import Context, integral

    with pytest.raises(GbError) as e:
        ctx.get(integral(99, "POLY", n=(8,)))
    assert e.value.code == 1
    with pytest.raises(GbError) as e:  # PROP1 needs a table
        ctx.get(integral("QLOOP", "PROP1", n=(8, 8), args=(0, 1.0, 1.0)), ())
    assert e.value.code == 1
    with pytest.raises(GbError) as e:
        ctx.get(integral("ANGLE", "POLY", n=(0, 8)))
    assert e.value.code == 1
    small = Context(0, budget_bytes=1024)
    try:
        w = subset(W, "C1")
        items, tabs = W.engine_items(w)
        t = small.table(*tabs[0])
        with pytest.raises(GbError) as e:
            small.batch(items, [t])
        assert e.value.code == 3
    finally:
        small.close()
