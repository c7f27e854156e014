"""Edge cases of the catalogue paths through the C ABI, against the FP64 oracle.

* extreme and ragged quadrature orders of the 3D family (workload C3's integrand): the largest
  order (256^3 = 16.8M points in one integral), the smallest, and phi orders 1 and 2 and odd /
  even mixes (the phi fold sums the first half of a symmetric rule with doubled weights and
  the middle node of an odd rule once);
* external momentum p = 0 (C1, C3);
* a NaN-filled dressing table poisons only the integrals that read it (per-item tables via
  table_base), in a batch with clean ones;
* an empty batch is an argument error (status code), not a launch.

Tolerances as in test_gpu_parity.py: FP64 1e-12, FP32C 1e-9.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-9


@pytest.fixture(scope="module")
def W():
    from diffrg_gb300 import workloads

    return workloads


def rel(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


def run(ctx, W, w, prec):
    items, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    b = ctx.batch(items, T, prec)
    out = b.get()
    b.close()
    for t in T:
        t.close()
    return out


C3_ORDERS = [(256, 256, 256), (16, 16, 16), (16, 256, 17), (33, 16, 1), (16, 40, 2), (255, 17, 3), (1, 1, 1),
             (64, 1, 64)]


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32c", TOL32), ("fp32f", 2e-8)])
def test_c3_extreme_and_ragged_orders(ctx, oracle, W, prec, tol):
    w = W.c3(8)
    w["orders"] = np.array(C3_ORDERS, dtype=np.int32)
    w["P"] = np.array([0.7, 0.01, 3.9, 0.0, 1.3, 0.2, 0.5, 2.0])
    got = run(ctx, W, w, prec)
    ref = W.oracle_values(w, oracle)
    err = rel(got, ref)
    print(prec, "C3 edge orders rel err", " ".join("%.2e" % e for e in err))
    assert np.all(np.isfinite(got))
    # The FP32-compensated form keeps each point within a few 1e-9 (the FP32 table fraction,
    # ~3e-8 of a cell, times the table's change over a cell); over an integral these errors
    # average out (~3e-11 on C3), but integrals of one or a few phi nodes keep them: those are
    # held to 5e-9, the others to the 1e-9 target.
    few = np.prod(w["orders"].astype(np.int64), axis=1) < 1024
    assert err[~few].max() <= tol
    assert err[few].max() <= {"fp32c": 5e-9, "fp32f": 1e-6}.get(prec, tol)  # fast form: FP32 per point


@pytest.mark.parametrize("prec,tol", [("fp64", TOL64), ("fp32c", TOL32)])
def test_zero_external_momentum(ctx, oracle, W, prec, tol):
    w = W.c1()
    w["p"] = np.array([0.0, 1e-3, 0.0, 2.0])
    got = run(ctx, W, w, prec)
    ref = W.oracle_values(w, oracle)
    assert rel(got, ref).max() <= tol
    assert got[0] == got[2]  # same integral, same bits


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_nan_table_poisons_only_its_items(ctx, oracle, W, prec):
    w = W.c1()
    w["p"] = w["p"][:4]
    spec, Z = w["tables"][0]
    Znan = np.full_like(Z, np.nan)
    items, _ = W.engine_items(w)
    # items 0 and 2 read the NaN table (table_base 0), items 1 and 3 the clean one (table_base 1)
    for i, g in enumerate(items):
        g.table_base = i % 2
    tn, tc = ctx.table(spec, Znan), ctx.table(spec, Z)
    b = ctx.batch(items, [tn, tc], prec)
    out = b.get()
    b.close()
    tn.close()
    tc.close()
    ref = W.oracle_values(w, oracle)
    assert np.isnan(out[0]) and np.isnan(out[2])
    tol = TOL64 if prec == "fp64" else TOL32
    assert rel(out[[1, 3]], ref[[1, 3]]).max() <= tol


def test_empty_batch_is_an_argument_error(ctx):
    from diffrg_gb300 import GbError

    with pytest.raises(GbError) as e:
        ctx.batch([], (), "fp32c")
    assert e.value.code == 1


def test_mixed_kinds_in_one_batch_are_bitwise_alone(ctx, W):
    """C2 (finite-T loop, mode-interpolated slices) and C5 (4D vertex, cos-axis slices) items in
    one batch, each reading its own tables through table_base: every result is bit-identical to
    the same integral alone, and within 1e-9 of the oracle."""
    from test_gpu_parity import subset

    w2, w5 = subset(W, "C2"), subset(W, "C5")
    i2, t2 = W.engine_items(w2)
    i5, t5 = W.engine_items(w5)
    for g in i5:
        g.table_base = 1
    T = [ctx.table(s, d) for s, d in t2 + t5]
    items = [g for pair in zip(i2, i5) for g in pair] + i2[len(i5):]
    b = ctx.batch(items, T, "fp32c")
    mix = b.get()
    b.close()
    for k in (0, 1, 2, 3, 11):
        b1 = ctx.batch([items[k]], T, "fp32c")
        alone = b1.get()[0]
        b1.close()
        assert alone == mix[k]
    got2 = np.concatenate([mix[0:2 * len(i5):2], mix[2 * len(i5):]])
    got5 = mix[1:2 * len(i5):2]
    assert rel(got2, W.oracle_values(w2, oracle_mod())).max() <= TOL32
    assert rel(got5, W.oracle_values(w5, oracle_mod())).max() <= TOL32
    for t in T:
        t.close()


def test_c5_small_q_order_falls_back_to_the_staged_table_kernel(ctx, oracle, W):
    """With few q nodes a work unit spans many cos1 nodes and their slices do not fit shared
    memory: the 4D vertex integrals then run on the kernel with the staged 2D tables, at the
    same accuracy."""
    w = W.c5()
    w["P"], w["alpha"] = w["P"][[0, 40, 127]], w["alpha"][[0, 40, 127]]
    w["n"] = (8, 64, 32, 16)
    got = run(ctx, W, w, "fp32c")
    ref = W.oracle_values(w, oracle)
    assert rel(got, ref).max() <= TOL32


def oracle_mod():
    from oracle import oracle as O

    O.build()
    return O


@pytest.mark.parametrize("spec_q", [(48, 0, 0.0, 5.0), (24, 1, 1e-3, 20.0)], ids=["linear", "coarse-log"])
def test_c2_tables_without_cell_reciprocals(ctx, oracle, W, spec_q):
    """Finite-T loop on dressing tables whose |q| axis is linear, or logarithmic with cells
    wider than the cell-centre reciprocals cover (54 %): the fraction comes from the
    double-float index instead, at the same 1e-9 (and 2e-8 for the fast form).  A linear |q|
    axis is fed the root of |q+p|^2, a log axis its square with half the scale."""
    from diffrg_gb300.workloads import spec_2d, seeded_table

    from test_gpu_parity import subset

    w = subset(W, "C2")
    n1, log1, lo1, hi1 = spec_q
    Z = seeded_table((n1, 64), 77).T.copy()
    w["tables"] = [(spec_2d(64, 0, 0.0, 64.0, n1, log1, lo1, hi1), Z)]
    ref = W.oracle_values(w, oracle)
    assert rel(run(ctx, W, w, "fp32c"), ref).max() <= TOL32
    assert rel(run(ctx, W, w, "fp32f"), ref).max() <= 2e-8  # the fast form's tolerance


def test_c5_tables_with_linear_momentum_axis(ctx, oracle, W):
    """4D vertex on 2D tables whose momentum axis is linear (no cell-centre reciprocals)."""
    from diffrg_gb300.workloads import spec_2d, seeded_table

    w = W.c5()
    w["P"], w["alpha"] = w["P"][[0, 63, 100]], w["alpha"][[0, 63, 100]]
    sp = spec_2d(200, 0, 0.0, 40.0, 48, 0, -1.0, 1.0)
    w["tables"] = [(sp, seeded_table((200, 48), 5, base=1.0, amp=0.5)),
                   (sp, seeded_table((200, 48), 6, base=0.5, amp=1.0))]
    ref = W.oracle_values(w, oracle)
    assert rel(run(ctx, W, w, "fp32c"), ref).max() <= TOL32
    assert rel(run(ctx, W, w, "fp32f"), ref).max() <= 2e-8  # the fast form (staged-table kernel)


def test_update_many_equals_single_updates(ctx, oracle, W):
    """gb_table_update_many: the same results as one gb_table_update per table, every epoch
    advanced once, and a table listed twice is an argument error."""
    from diffrg_gb300 import GbError
    from test_gpu_parity import subset

    w = subset(W, "C3")
    items, tabs = W.engine_items(w)
    T = [ctx.table(s, d) for s, d in tabs]
    rng = np.random.default_rng(11)
    new = [d * (1 + 0.1 * rng.random(d.shape)).astype(np.float32) for _, d in tabs]
    e0 = [t.epoch for t in T]
    ctx.update_tables(zip(T, new))
    assert [t.epoch for t in T] == [e + 1 for e in e0]
    b = ctx.batch(items, T, "fp32c")
    many = b.get()
    b.close()
    for t, d in zip(T, [d for _, d in tabs]):
        t.update(d)
    for t, d in zip(T, new):
        t.update(d)
    b = ctx.batch(items, T, "fp32c")
    single = b.get()
    b.close()
    assert np.array_equal(many, single)
    w2 = dict(w)
    w2["tables"] = [(s, d) for (s, _), d in zip(tabs, new)]
    assert rel(many, W.oracle_values(w2, oracle)).max() <= TOL32
    with pytest.raises(GbError) as e:
        ctx.update_tables([(T[0], new[0]), (T[0], new[0])])
    assert e.value.code == 1
    for t in T:
        t.close()
