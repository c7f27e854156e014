"""C4: a flow of 32 dressing functions on 128 external momenta, integrated in RG time with an
embedded Runge-Kutta 4(5) pair (Cash-Karp, the stepper DiFfRG takes from boost odeint,
DiFfRG/include/DiFfRG/timestepping/boost_rk.hh:21), whose right-hand side is served by the
library's request loop.

Every right-hand-side evaluation publishes the current dressing functions as device tables
(one 128-point log-spaced FP32 table per function, x = p^2 in [1e-4, 100]) and asks for the
4096 loop integrals I_i(p_j) as requests of 8..2048 integrals (sizes log-uniform, seeded).
Even-numbered functions use a 2D loop (IntegratorAngle measure, d = 4, orders (x, cos)) with
the PROP1 integrand on table i; odd-numbered ones a 3D loop (Integrator3D measure, orders
(x, cos, phi)) with PROP3 on tables i..i+3 (cyclic).  Orders are drawn once per function
from 32..128 per axis.  Requests arrive as a Poisson process whose mean integral rate is
`rate` (2000 integrals/s by default; rate=None submits a whole evaluation at once, the
saturated case).  The flow itself is synthetic:
    dZ_i(p_j)/dt = -(Z_i(p_j) - 1)/2 + I_i(p_j) / (4 max_j |I_i(p_j)|),   k = exp(-t),
which keeps every Z_i in [0.5, 1.5] so that the propagators stay finite.
"""
from __future__ import annotations

import math
import time

import numpy as np

from .engine import Context, Table, integral, integral_array, integral_view
from .workloads import SEEDS, seeded_table, spec_log

N_FUNC = 32
N_P = 128
X_LO, X_HI = 1e-4, 100.0
THETA = 1.0  # external angle of the 3D loops

# Cash-Karp tableau (J. R. Cash, A. H. Karp, ACM TOMS 16 (1990) 201)
CK_C = (0.0, 1 / 5, 3 / 10, 3 / 5, 1.0, 7 / 8)
CK_A = ((),
        (1 / 5,),
        (3 / 40, 9 / 40),
        (3 / 10, -9 / 10, 6 / 5),
        (-11 / 54, 5 / 2, -70 / 27, 35 / 27),
        (1631 / 55296, 175 / 512, 575 / 13824, 44275 / 110592, 253 / 4096))
CK_B5 = (37 / 378, 0.0, 250 / 621, 125 / 594, 0.0, 512 / 1771)
CK_B4 = (2825 / 27648, 0.0, 18575 / 48384, 13525 / 55296, 277 / 14336, 1 / 4)


def c4(seed: int = SEEDS["C4"]) -> dict:
    rng = np.random.default_rng(seed)
    funcs = []
    for i in range(N_FUNC):
        dim = 2 if i % 2 == 0 else 3
        funcs.append({"dim": dim, "orders": tuple(int(v) for v in rng.integers(32, 129, size=dim))})
    x = np.logspace(math.log10(X_LO), math.log10(X_HI), N_P)
    y0 = seeded_table((N_P, N_FUNC), seed + 1, base=0.95, amp=0.1).T.astype(np.float64)
    pts = sum(int(np.prod(f["orders"])) for f in funcs) * N_P
    return {"name": "C4", "funcs": funcs, "x": x, "p": np.sqrt(x), "y0": y0, "spec": spec_log(N_P, X_LO, X_HI),
            "x_extent": 4.0, "rate": 2000.0, "size_lo": 8, "size_hi": 2048,
            "integrals_per_rhs": N_FUNC * N_P, "points_per_rhs": pts}


def table_order():
    """Indices of the table list passed with every request: 0..31 then 0, 1, 2, so that the
    four tables of 3D function i are the contiguous list entries i..i+3."""
    return list(range(N_FUNC)) + [0, 1, 2]


class RhsItems:
    """The right-hand side's descriptors as one ctypes array, built once; at(k) rewrites the
    RG scale of every descriptor in place (a numpy view of the array)."""

    def __init__(self, w: dict):
        self.arr = integral_array(rhs_items(w, 1.0))
        self.view = np.ctypeslib.as_array(self.arr)

    def at(self, k: float):
        self.view["k"][:] = k
        return self.arr

    def slice(self, lo: int, hi: int):
        return integral_view(self.arr, lo, hi)


def rhs_items(w: dict, k: float):
    """The N_FUNC * N_P integral descriptors of one right-hand side, row-major in (i, j)."""
    items = []
    ct, st = math.cos(THETA), math.sin(THETA)
    for i, f in enumerate(w["funcs"]):
        for pj in w["p"]:
            if f["dim"] == 2:
                items.append(integral("ANGLE", "PROP1", d=4, n=f["orders"], k=k, x_extent=w["x_extent"],
                                      args=(0.0, pj, 1.0), table_base=i))
            else:
                items.append(integral("3D", "PROP3", n=f["orders"], k=k, x_extent=w["x_extent"],
                                      args=(0.0, pj, ct, st), table_base=i))
    return items


def request_sizes(rng, total: int, lo: int, hi: int):
    """Request sizes log-uniform in [lo, hi] covering `total` integrals (the last one is cut)."""
    sizes = []
    left = total
    while left > 0:
        s = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        s = max(lo, min(hi, s, left))
        if left - s < lo and left - s > 0:
            s = left if left <= hi else s
        sizes.append(min(s, left))
        left -= sizes[-1]
    return sizes


def mean_request_size(lo: int, hi: int) -> float:
    return (hi - lo) / math.log(hi / lo)


class Flow:
    """The C4 system on one context, its right-hand side served by the request loop."""

    def __init__(self, ctx: Context, w: dict | None = None, precision: str = "fp32c", rate: float | None = 2000.0,
                 seed: int = SEEDS["C4"] + 7):
        self.ctx = ctx
        self.w = w or c4()
        self.precision = precision
        self.rate = rate
        self.rng = np.random.default_rng(seed)
        self.tables = [Table(ctx, self.w["spec"], self.w["y0"][i]) for i in range(N_FUNC)]
        self.tlist = [self.tables[i] for i in table_order()]
        self.items = RhsItems(self.w)
        self.rhs_evals = 0
        self.requests = 0
        self.integrals = 0

    def close(self):
        for t in self.tables:
            t.close()

    def integrals_at(self, t: float, y: np.ndarray) -> np.ndarray:
        """Publish y as the tables and serve all N_FUNC x N_P integrals at RG time t."""
        self.ctx.update_tables([(self.tables[i], y[i]) for i in range(N_FUNC)])
        n = self.w["integrals_per_rhs"]
        self.items.at(math.exp(-t))
        sizes = request_sizes(self.rng, n, self.w["size_lo"], self.w["size_hi"])
        tickets = []
        off = 0
        t_next = time.perf_counter()
        lam = None if not self.rate else self.rate / mean_request_size(self.w["size_lo"], self.w["size_hi"])
        for s in sizes:
            if lam:
                t_next += self.rng.exponential(1.0 / lam)
                dt = t_next - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
            tickets.append((off, self.ctx.submit(self.items.slice(off, off + s), self.tlist, self.precision)))
            off += s
        out = np.empty(n)
        for o, tk in tickets:
            out[o:o + tk.n] = tk.wait()
        self.rhs_evals += 1
        self.requests += len(sizes)
        self.integrals += n
        return out.reshape(N_FUNC, N_P)

    def rhs(self, t: float, y: np.ndarray) -> np.ndarray:
        I = self.integrals_at(t, y)
        scale = np.max(np.abs(I), axis=1, keepdims=True)
        scale[scale == 0] = 1.0
        return -0.5 * (y - 1.0) + 0.25 * I / scale

    def integrate(self, t0: float, t1: float, h0: float = 0.25, rtol: float = 1e-6, atol: float = 1e-9,
                  max_steps: int = 1000):
        """Adaptive Cash-Karp from t0 to t1 starting at y0; (y(t1), accepted, rejected)."""
        return integrate_adaptive(self.rhs, self.w["y0"].copy(), t0, t1, h0, rtol, atol, max_steps)


def cash_karp_step(rhs, t: float, y: np.ndarray, h: float):
    """One Cash-Karp step of y' = rhs(t, y): (5th-order solution, embedded error estimate)."""
    ks = []
    for s in range(6):
        ys = y.copy()
        for a, kk in zip(CK_A[s], ks):
            ys = ys + h * a * kk
        ks.append(rhs(t + CK_C[s] * h, ys))
    y5 = y + h * sum(b * kk for b, kk in zip(CK_B5, ks))
    err = h * sum((b5 - b4) * kk for b5, b4, kk in zip(CK_B5, CK_B4, ks))
    return y5, err


def integrate_adaptive(rhs, y0, t0: float, t1: float, h0: float = 0.25, rtol: float = 1e-6, atol: float = 1e-9,
                       max_steps: int = 1000):
    """Adaptive Cash-Karp integration with a standard step-size controller:
    err = max |e| / (atol + rtol |y|), accept at err <= 1, growth <= 5x, shrink >= 0.1x."""
    t, y, h = t0, np.array(y0, dtype=np.float64), h0
    acc = rej = 0
    while t < t1 - 1e-12 and acc + rej < max_steps:
        h = min(h, t1 - t)
        y5, err = cash_karp_step(rhs, t, y, h)
        e = float(np.max(np.abs(err) / (atol + rtol * np.abs(y))))
        if e <= 1.0:
            t, y = t + h, y5
            acc += 1
            h *= min(5.0, 0.9 * e ** -0.2) if e > 0 else 5.0
        else:
            rej += 1
            h *= max(0.1, 0.9 * e ** -0.25)
    return y, acc, rej


def oracle_subset(O, w: dict, y: np.ndarray, k: float, pairs):
    """FP64 oracle values of the integrals (i, j) in `pairs` for tables y and scale k."""
    spec = w["spec"]
    out = []
    ct, st = math.cos(THETA), math.sin(THETA)
    for i, j in pairs:
        f = w["funcs"][i]
        pj = w["p"][j]
        args = np.zeros((1, 24))
        args[0, 1] = pj
        if f["dim"] == 2:
            args[0, 2] = 1.0
            d = O.family_desc("ANGLE", n=f["orders"], d=4, x_extent=w["x_extent"])
            tabs = [(spec, y[i].astype(np.float32))]
            out.append(O.family(d, "PROP1", k, args, tables=tabs)[0])
        else:
            args[0, 2] = ct
            args[0, 3] = st
            d = O.family_desc("3D", n=f["orders"], x_extent=w["x_extent"])
            tabs = [(spec, y[(i + m) % N_FUNC].astype(np.float32)) for m in range(4)]
            out.append(O.family(d, "PROP3", k, args, tables=tabs)[0])
    return np.array(out)
