"""Seeded synthetic workloads C1-C5 of the momentum-loop integration benchmark.

Every dressing-function table is FP32 (the reference's TexLinearInterpolator* store
``float`` data, DiFfRG/src/DiFfRG/physics/interpolation/tex_linear_interpolation_1D.cu:40-64),
so the engine and the FP64 oracle read the very same numbers.  Values are
``base + amp * u``, u ~ U[0,1) from ``numpy.random.default_rng(seed)`` (PCG64), smoothed by a
5-point moving average along the first (momentum) axis; at the two ends the window shrinks
to the points that exist (3 or 4 points).

C1  d=4 loop: 64 p log-spaced in [1e-3,10]; q in [0,2] (64 GL in q) x cos (32 GL);
    Z: 128 log-spaced points in [1e-4,100].
C2  finite-T 3+1D: T in {0.05,0.2,1.0} x 128 p; n=-64..64; q 64 GL x cos 32 GL;
    Z(|w_n|/(2 pi T), |q|): 64 (linear in mode index on [0,64]) x 128 (log |q| in [1e-3,20]).
C3  4096 uneven 3D (x, cos, phi) loops (Integrator3D measure, x_extent=4, k=1); GL orders
    round(exp(U[ln16, ln256])) per axis; |p| log-uniform in [1e-2,4], external angle 1 rad;
    tables A,B,C,D: 256 log-spaced points in [1e-4,100].
C4  serving: see diffrg_gb300.serving.
C5  4D vertex: 64 |p| log-spaced in [1e-2,4] x angle in {pi/3, pi/2}; Integrator4D measure
    with (x, cos1, cos2, phi) = (128, 64, 32, 16) GL, x_extent=4, k=1; two 256x64 FP32 tables
    (log x in [1e-4,100]) x (linear t in [-1,1]), bilinear.
"""
from __future__ import annotations

import math

import numpy as np

SEEDS = {"C1_Z": 1001, "C2_Z": 1002, "C3_A": 1003, "C3_B": 1004, "C3_C": 1005, "C3_D": 1006,
         "C3_orders": 1007, "C3_p": 1008, "C5_A": 1009, "C5_B": 1010, "C4": 1011}


def smooth5(u: np.ndarray, axis: int = 0) -> np.ndarray:
    """5-point moving average along `axis`, window shrunk at the edges."""
    u = np.moveaxis(np.asarray(u, dtype=np.float64), axis, 0)
    n = u.shape[0]
    out = np.empty_like(u)
    for i in range(n):
        lo, hi = max(0, i - 2), min(n, i + 3)
        out[i] = u[lo:hi].mean(axis=0)
    return np.moveaxis(out, 0, axis)


def seeded_table(shape, seed, base=1.0, amp=0.5) -> np.ndarray:
    rng = np.random.default_rng(seed)
    u = rng.random(shape)
    return (base + amp * smooth5(u, axis=0)).astype(np.float32)


def spec_log(n, lo, hi):
    return {"n0": n, "log0": 1, "lo0": float(lo), "hi0": float(hi)}


def spec_2d(n0, log0, lo0, hi0, n1, log1, lo1, hi1):
    return {"n0": n0, "log0": int(log0), "lo0": float(lo0), "hi0": float(hi0),
            "n1": n1, "log1": int(log1), "lo1": float(lo1), "hi1": float(hi1)}


def c1():
    Z = seeded_table((128,), SEEDS["C1_Z"])
    p = np.logspace(-3, 1, 64)
    return {"name": "C1", "tables": [(spec_log(128, 1e-4, 100.0), Z)], "p": p, "nq": 64, "nc": 32, "qmax": 2.0,
            "points_per_integral": 64 * 32}


def c2():
    Z = seeded_table((128, 64), SEEDS["C2_Z"]).T.copy()  # smooth along |q| (128), store (mode, |q|)
    Ts = np.array([0.05, 0.2, 1.0])
    p = np.logspace(-3, 1, 128)
    PP, TT = np.meshgrid(p, Ts)
    return {"name": "C2", "tables": [(spec_2d(64, 0, 0.0, 64.0, 128, 1, 1e-3, 20.0), Z)],
            "p": PP.ravel().copy(), "T": TT.ravel().copy(), "M": 64, "nq": 64, "nc": 32, "qmax": 2.0,
            "points_per_integral": 129 * 64 * 32}


def c3(n_integrals=4096):
    tabs = [(spec_log(256, 1e-4, 100.0), seeded_table((256,), SEEDS[k])) for k in ("C3_A", "C3_B", "C3_C", "C3_D")]
    rng = np.random.default_rng(SEEDS["C3_orders"])
    orders = np.rint(np.exp(rng.uniform(math.log(16), math.log(256), size=(n_integrals, 3)))).astype(np.int32)
    rngp = np.random.default_rng(SEEDS["C3_p"])
    P = np.exp(rngp.uniform(math.log(1e-2), math.log(4.0), size=n_integrals))
    theta = 1.0
    return {"name": "C3", "tables": tabs, "orders": orders, "P": P, "cos_t": math.cos(theta),
            "sin_t": math.sin(theta), "x_extent": 4.0, "k": 1.0,
            "points": int(np.prod(orders.astype(np.int64), axis=1).sum())}


def c5():
    A = seeded_table((256, 64), SEEDS["C5_A"], base=1.0, amp=0.5)
    B = seeded_table((256, 64), SEEDS["C5_B"], base=0.5, amp=1.0)
    sp = spec_2d(256, 1, 1e-4, 100.0, 64, 0, -1.0, 1.0)
    P = np.logspace(-2, math.log10(4.0), 64)
    alphas = np.array([math.pi / 3, math.pi / 2])
    PP, AA = np.meshgrid(P, alphas, indexing="ij")
    return {"name": "C5", "tables": [(sp, A), (sp, B)], "P": PP.ravel().copy(), "alpha": AA.ravel().copy(),
            "n": (128, 64, 32, 16), "x_extent": 4.0, "k": 1.0, "points_per_integral": 128 * 64 * 32 * 16}


def poly_args(c=0.0, q=(1, 0, 0, 0, 0, 0), a1=(1, 0, 0, 0), a2=(1, 0, 0, 0), a3=(1, 0, 0, 0), t=(1, 0, 0, 0)):
    """Argument vector (24 slots) of the polynomial KAT integrand:
    [c, q0..q5, a1_0..3, a2_0..3, a3_0..3, t0..3, pad]."""
    a = np.zeros(24)
    a[0] = c
    a[1:7] = q
    a[7:11] = a1
    a[11:15] = a2
    a[15:19] = a3
    a[19:23] = t
    return a


# ---------------------------------------------------------------------------------------------
# Engine descriptors of the workloads (gb_integral lists + table lists)
# ---------------------------------------------------------------------------------------------
def engine_items(w):
    """(list of gb_integral descriptors, list of (spec, data) tables) for workload dict `w`."""
    from .engine import integral

    name = w["name"]
    if name == "C1":
        items = [integral("QLOOP", "PROP1", n=(w["nq"], w["nc"]), k=1.0, x_extent=w["qmax"], args=(0.0, p, 1.0))
                 for p in w["p"]]
    elif name == "C2":
        items = [integral("QLOOP_T", "FTLOOP", n=(w["nq"], w["nc"]), k=1.0, x_extent=w["qmax"], x0_summands=w["M"],
                          T=T, args=(0.0, p, T, 0.0)) for p, T in zip(w["p"], w["T"])]
    elif name == "C3":
        items = [integral("3D", "PROP3", n=tuple(int(v) for v in o), k=w["k"], x_extent=w["x_extent"],
                          args=(0.0, P, w["cos_t"], w["sin_t"])) for o, P in zip(w["orders"], w["P"])]
    elif name == "C5":
        items = [integral("4D", "VERT4", n=w["n"], k=w["k"], x_extent=w["x_extent"],
                          args=(0.0, P, math.cos(a), math.sin(a))) for P, a in zip(w["P"], w["alpha"])]
    else:
        raise ValueError(name)
    return items, w["tables"]


def oracle_values(w, oracle_mod, threads=0, subset=None):
    """FP64 oracle values of workload `w` (optionally only the integrals in `subset`)."""
    O = oracle_mod
    name = w["name"]
    idx = np.arange(len(w["P"] if "P" in w else w["p"])) if subset is None else np.asarray(subset)
    if name == "C1":
        return O.w1(w["tables"][0], w["nq"], w["nc"], w["qmax"], w["p"][idx], threads=threads)
    if name == "C2":
        return O.w2(w["tables"][0], w["M"], w["nq"], w["nc"], w["qmax"], w["p"][idx], w["T"][idx], threads=threads)
    if name == "C3":
        descs = [O.family_desc("3D", n=tuple(int(v) for v in w["orders"][i]), x_extent=w["x_extent"]) for i in idx]
        args = np.zeros((idx.size, 24))
        args[:, 1] = w["P"][idx]
        args[:, 2] = w["cos_t"]
        args[:, 3] = w["sin_t"]
        return O.family(descs, "PROP3", w["k"], args, tables=w["tables"], threads=threads)
    if name == "C5":
        d = O.family_desc("4D", n=w["n"], x_extent=w["x_extent"])
        args = np.zeros((idx.size, 24))
        args[:, 1] = w["P"][idx]
        args[:, 2] = np.cos(w["alpha"][idx])
        args[:, 3] = np.sin(w["alpha"][idx])
        return O.family(d, "VERT4", w["k"], args, tables=w["tables"], threads=threads)
    raise ValueError(name)
