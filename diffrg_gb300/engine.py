"""Python host API above the C ABI (libgbint.so).

Mirrors the reference objects a flow-equation code touches on the integration path:
``QuadratureProvider`` (``Context.gl`` / ``Context.matsubara``), dressing-function tables
(``Table``; TexLinearInterpolator* in the reference), one integrator evaluation
(``Context.get``) and the fan-out of many integrals (``Batch``; request_data/update_data in
DiFfRG/include/DiFfRG/physics/utils.hh:115-147).  Errors raise ``GbError`` like the reference
throws std::runtime_error.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import capi
from .capi import FAM, IG, PREC, GbError, Integral, TableSpec


def integral(family, integrand="POLY", n=(0, 0, 0, 0), k=1.0, d=4, x_extent=1.0, x0_extent=0.0, x0_summands=0,
             T=0.0, E=0.0, qmin=(-np.pi,) * 3, qmax=(np.pi,) * 3, args=(), table_base=0) -> Integral:
    """Descriptor of one integral (gb_integral); it reads tables[table_base:] of its batch."""
    g = Integral()
    g.family = FAM[family] if isinstance(family, str) else int(family)
    g.integrand = IG[integrand] if isinstance(integrand, str) else int(integrand)
    g.d = d
    nn = list(n) + [0] * (4 - len(n))
    for i in range(4):
        g.n[i] = int(nn[i])
    g.table_base = int(table_base)
    g.x_extent = x_extent
    g.x0_extent = x0_extent
    g.x0_summands = int(x0_summands)
    g.T = T
    g.E = E
    g.k = k
    for i in range(3):
        g.qmin[i] = qmin[i]
        g.qmax[i] = qmax[i]
    a = np.zeros(capi.GB_MAX_ARGS)
    a[:len(args)] = args
    for i in range(capi.GB_MAX_ARGS):
        g.args[i] = float(a[i])
    return g


class Table:
    def __init__(self, ctx: "Context", spec: dict, data=None):
        self.ctx = ctx
        self.spec = dict(spec)
        s = TableSpec(spec["n0"], int(spec["log0"]), spec["lo0"], spec["hi0"], spec.get("n1", 0),
                      int(spec.get("log1", 0)), spec.get("lo1", 0.0), spec.get("hi1", 1.0))
        h = C.c_void_p()
        ctx.check(capi.lib().gb_table_create(ctx.h, C.byref(s), C.byref(h)))
        self.h = h
        self.shape = (spec["n0"],) if not spec.get("n1") else (spec["n0"], spec["n1"])
        if data is not None:
            self.update(data)

    def update(self, data, stream=None):
        d = np.ascontiguousarray(data, dtype=np.float32)
        if d.size != int(np.prod(self.shape)):
            raise ValueError("table data has %d values, expected %s" % (d.size, self.shape))
        self.ctx.check(capi.lib().gb_table_update(self.ctx.h, self.h, d.ctypes.data_as(C.POINTER(C.c_float)),
                                                   C.c_void_p(stream) if stream else None))

    @property
    def epoch(self) -> int:
        e = C.c_uint64()
        self.ctx.check(capi.lib().gb_table_epoch(self.ctx.h, self.h, C.byref(e)))
        return int(e.value)

    def close(self):
        if self.h:
            capi.lib().gb_table_destroy(self.ctx.h, self.h)
            self.h = None


def integral_array(integrals) -> "C.Array":
    """A ctypes array of gb_integral: `integrals` itself if it already is one (no copy)."""
    if isinstance(integrals, C.Array):
        return integrals
    return (Integral * len(integrals))(*integrals)


def integral_view(arr: "C.Array", lo: int, hi: int) -> "C.Array":
    """Elements lo..hi-1 of a ctypes gb_integral array, sharing its memory."""
    if not 0 <= lo <= hi <= len(arr):
        raise IndexError("integral_view out of range")
    return (Integral * (hi - lo)).from_address(C.addressof(arr) + lo * C.sizeof(Integral))


def _table_array(tables: Sequence[Table]):
    arr = (C.c_void_p * max(1, len(tables)))()
    for i, t in enumerate(tables):
        arr[i] = t.h
    return arr


class Batch:
    def __init__(self, ctx: "Context", integrals: Sequence[Integral], tables: Sequence[Table] = (),
                 precision: str = "fp32c"):
        self.ctx = ctx
        self.n = len(integrals)
        arr = integral_array(integrals)
        h = C.c_void_p()
        ctx.check(capi.lib().gb_batch_create(ctx.h, arr, self.n, _table_array(tables), len(tables),
                                             PREC[precision], C.byref(h)))
        self.h = h
        self.tables = list(tables)
        self.precision = precision
        pts = C.c_uint64()
        nu = C.c_int()
        ni = C.c_int()
        ctx.check(capi.lib().gb_batch_info(ctx.h, h, C.byref(pts), C.byref(nu), C.byref(ni)))
        self.points = int(pts.value)
        self.n_units = int(nu.value)

    def run(self, stream=None, d_out=None):
        self.ctx.check(capi.lib().gb_batch_run(self.ctx.h, self.h, C.c_void_p(d_out) if d_out else None,
                                               C.c_void_p(stream) if stream else None))

    def run_graph(self, stream=None):
        self.ctx.check(capi.lib().gb_batch_run_graph(self.ctx.h, self.h, C.c_void_p(stream) if stream else None))

    def results(self, stream=None) -> np.ndarray:
        out = np.zeros(self.n)
        self.ctx.check(capi.lib().gb_batch_results(self.ctx.h, self.h, capi._dp(out),
                                                   C.c_void_p(stream) if stream else None))
        return out

    def get(self, stream=None) -> np.ndarray:
        out = np.zeros(self.n)
        self.ctx.check(capi.lib().gb_batch_get(self.ctx.h, self.h, capi._dp(out),
                                               C.c_void_p(stream) if stream else None))
        return out

    def run_plain(self, n_streams=16) -> np.ndarray:
        out = np.zeros(self.n)
        self.ctx.check(capi.lib().gb_batch_run_plain(self.ctx.h, self.h, capi._dp(out), n_streams))
        return out

    def close(self):
        if self.h:
            capi.lib().gb_batch_destroy(self.ctx.h, self.h)
            self.h = None


class Graph:
    """A captured sweep (gb_graph): replay() launches every captured batch run at once."""

    def __init__(self, ctx: "Context", h):
        self.ctx = ctx
        self.h = h
        n = C.c_int()
        ctx.check(capi.lib().gb_graph_info(ctx.h, h, C.byref(n)))
        self.kernel_launches = n.value

    def replay(self, stream=None):
        self.ctx.check(capi.lib().gb_graph_launch(self.ctx.h, self.h, C.c_void_p(stream) if stream else None))

    def close(self):
        if self.h:
            capi.lib().gb_graph_destroy(self.ctx.h, self.h)
            self.h = None


class Ticket:
    """A submitted request: poll() / wait() return its results (float64, one per integral)."""

    def __init__(self, ctx: "Context", tid: int, n: int):
        self.ctx = ctx
        self.id = tid
        self.n = n

    def poll(self):
        """The results if the request is finished, else None."""
        out = np.zeros(self.n)
        rc = capi.lib().gb_poll(self.ctx.h, self.id, capi._dp(out))
        if rc == capi.GB_EAGAIN:
            return None
        self.ctx.check(rc)
        return out

    def wait(self, timeout: float = 0.0) -> np.ndarray:
        out = np.zeros(self.n)
        self.ctx.check(capi.lib().gb_wait(self.ctx.h, self.id, capi._dp(out), timeout))
        return out

    def cancel(self) -> bool:
        """True if the request was still queued and is now canceled."""
        rc = capi.lib().gb_cancel(self.ctx.h, self.id)
        if rc == capi.GB_EAGAIN:
            return False
        self.ctx.check(rc)
        return True


# QuadratureType (DiFfRG/include/DiFfRG/common/quadrature/quadrature.hh:47)
QUAD_LEGENDRE, QUAD_CHEBYSHEV, QUAD_LAGUERRE, QUAD_HERMITE, QUAD_JACOBI = 0, 1, 2, 3, 4


def quad_rule_host(qtype: int, order: int):
    """Nodes and weights of a QuadratureType without a context (host only, no GPU)."""
    x = np.zeros(order)
    w = np.zeros(order)
    rc = capi.lib().gb_quad_rule_host(qtype, order, x.ctypes.data_as(C.POINTER(C.c_double)),
                                      w.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        raise GbError(rc, "gb_quad_rule_host(%d, %d)" % (qtype, order))
    return x, w


class Context:
    """One device context (gb_ctx): provider caches, node pool, table directory, streams."""

    def __init__(self, device: int = 0, budget_bytes: int = 0):
        L = capi.load()
        h = C.c_void_p()
        rc = L.gb_ctx_create(device, budget_bytes, C.byref(h))
        if rc != 0:
            raise GbError(rc, "gb_ctx_create(device=%d)" % device)
        self.h = h

    def last_error(self) -> str:
        buf = C.create_string_buffer(512)
        capi.lib().gb_last_error(self.h, buf, 512)
        return buf.value.decode()

    def check(self, rc: int):
        if rc != 0:
            raise GbError(rc, self.last_error())

    # QuadratureProvider
    def gl(self, order: int):
        hx = C.POINTER(C.c_double)()
        hw = C.POINTER(C.c_double)()
        self.check(capi.lib().gb_quad_gl(self.h, order, 0, C.byref(hx), C.byref(hw), None, None))
        return np.ctypeslib.as_array(hx, (order,)).copy(), np.ctypeslib.as_array(hw, (order,)).copy()

    def gl_device(self, order: int, dtype=0):
        dx = C.c_void_p()
        dw = C.c_void_p()
        self.check(capi.lib().gb_quad_gl(self.h, order, dtype, None, None, C.byref(dx), C.byref(dw)))
        return dx.value, dw.value

    def rule(self, qtype: int, order: int):
        """Host nodes and weights of a QuadratureType (QUAD_* below) from the context's cache."""
        hx = C.POINTER(C.c_double)()
        hw = C.POINTER(C.c_double)()
        self.check(capi.lib().gb_quad_rule(self.h, qtype, order, 0, C.byref(hx), C.byref(hw), None, None))
        return np.ctypeslib.as_array(hx, (order,)).copy(), np.ctypeslib.as_array(hw, (order,)).copy()

    def rule_device(self, qtype: int, order: int, dtype=0):
        dx = C.c_void_p()
        dw = C.c_void_p()
        self.check(capi.lib().gb_quad_rule(self.h, qtype, order, dtype, None, None, C.byref(dx), C.byref(dw)))
        return dx.value, dw.value

    def matsubara(self, T: float, E: float):
        n = C.c_int()
        hx = C.POINTER(C.c_double)()
        hw = C.POINTER(C.c_double)()
        tr = C.c_double()
        self.check(capi.lib().gb_quad_matsubara(self.h, T, E, 0, C.byref(n), C.byref(hx), C.byref(hw), None, None,
                                                C.byref(tr)))
        m = n.value
        return np.ctypeslib.as_array(hx, (m,)).copy(), np.ctypeslib.as_array(hw, (m,)).copy(), tr.value

    def quad_config(self, min_matsubara_size=32, vacuum_quad_size=48, add_matsubara_size=0):
        self.check(capi.lib().gb_quad_config(self.h, min_matsubara_size, vacuum_quad_size, add_matsubara_size))

    def table(self, spec: dict, data=None) -> Table:
        return Table(self, spec, data)

    def update_tables(self, pairs, stream=None):
        """Update several tables as one group (gb_table_update_many): served requests see all of
        them or none."""
        pairs = list(pairs)
        arrs = []
        for t, data in pairs:
            d = np.ascontiguousarray(data, dtype=np.float32)
            if d.size != int(np.prod(t.shape)):
                raise ValueError("table data has %d values, expected %s" % (d.size, t.shape))
            arrs.append(d)
        n = len(pairs)
        handles = (C.c_void_p * n)(*[t.h for t, _ in pairs])
        ptrs = (C.POINTER(C.c_float) * n)(*[d.ctypes.data_as(C.POINTER(C.c_float)) for d in arrs])
        self.check(capi.lib().gb_table_update_many(self.h, n, handles, ptrs, C.c_void_p(stream) if stream else None))

    def batch(self, integrals, tables=(), precision="fp32c") -> Batch:
        return Batch(self, integrals, tables, precision)

    def get(self, g: Integral, tables=(), precision="fp64") -> float:
        out = C.c_double()
        self.check(capi.lib().gb_get(self.h, C.byref(g), _table_array(tables), len(tables), PREC[precision],
                                     C.byref(out)))
        return out.value

    # autotuner
    def autotune(self, integrals, tables=(), precision="fp32c", cache_path=None, refresh=False) -> dict:
        """Time the work-unit schedules of the FP32-compensated kernels on these integrals (CTA
        width, rows per thread, inner split, unit order; one parameter at a time) and keep the
        fastest per kernel kind (batches created afterwards use them).  Returns {slot: threads}
        for the slots whose width is set; tune_report() has every measurement."""
        arr = integral_array(integrals)
        chosen = (C.c_int * 16)()
        self.check(capi.lib().gb_autotune(self.h, arr, len(arr), _table_array(tables), len(tables), PREC[precision],
                                          cache_path.encode() if cache_path else None, 1 if refresh else 0, chosen))
        return {k: chosen[k] for k in range(16) if chosen[k]}

    def tune_set(self, slot: int, threads: int):
        self.check(capi.lib().gb_tune_set(self.h, slot, threads))

    def tune_set_schedule(self, slot: int, threads=0, rows_per_thread=0, inner_split=0, unit_order="item"):
        sc = capi.Schedule(threads, rows_per_thread, inner_split,
                           capi.GB_ORDER_COST if unit_order == "cost" else capi.GB_ORDER_ITEM)
        self.check(capi.lib().gb_tune_set_schedule(self.h, slot, C.byref(sc)))

    def tune_get_schedule(self, slot: int) -> dict:
        sc = capi.Schedule()
        self.check(capi.lib().gb_tune_get_schedule(self.h, slot, C.byref(sc)))
        return {"threads": sc.threads, "rows_per_thread": sc.rows_per_thread, "inner_split": sc.inner_split,
                "unit_order": "cost" if sc.unit_order == capi.GB_ORDER_COST else "item"}

    def tune_report(self) -> dict:
        """The last autotune's measurements: per kind slot the default and chosen schedules with
        their median ms and every candidate's ms, parameter by parameter."""
        import json

        n = C.c_size_t()
        self.check(capi.lib().gb_tune_report(self.h, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value + 1)
        self.check(capi.lib().gb_tune_report(self.h, buf, n.value + 1, C.byref(n)))
        return json.loads(buf.value.decode())

    # CUDA-graph sweeps
    def capture(self, body, stream=None) -> Graph:
        """Capture body() -- gb_batch_run calls on `stream` (None: the context's stream) --
        into a replayable graph."""
        L = capi.lib()
        sp = C.c_void_p(stream) if stream else None
        self.check(L.gb_graph_capture_begin(self.h, sp))
        g = C.c_void_p()
        try:
            body()
        finally:
            rc = L.gb_graph_capture_end(self.h, sp, C.byref(g))
        self.check(rc)
        return Graph(self, g)

    # serving (continuous batching)
    def serve_start(self, max_inflight: int = 8, max_items: int = 2048):
        """Start the request loop: up to `max_inflight` device batches in flight, each merging
        queued requests up to `max_items` integrals."""
        self.check(capi.lib().gb_serve_start(self.h, max_inflight, max_items))

    def serve_start_device(self, ring_slots: int = 16, max_items: int = 2048, max_units: int = 1 << 21,
                           idle_seconds: float = 5e-3):
        """The device-resident request loop (gb_serve_start_device): gb_submit / Ticket.wait then
        go through a ring the GPU's persistent loop kernel reads; FP64 results."""
        self.check(capi.lib().gb_serve_start_device(self.h, ring_slots, max_items, max_units, idle_seconds))

    def device_loop_info(self) -> dict:
        """{"launches", "idle_exits", "running"} of the device-resident request loop."""
        la, ex, ru = C.c_longlong(), C.c_int(), C.c_int()
        self.check(capi.lib().gb_serve_device_info(self.h, C.byref(la), C.byref(ex), C.byref(ru)))
        return {"launches": la.value, "idle_exits": ex.value, "running": bool(ru.value)}

    def serve_stop(self):
        self.check(capi.lib().gb_serve_stop(self.h))

    def submit(self, integrals: Sequence[Integral], tables: Sequence[Table] = (), precision: str = "fp32c") -> "Ticket":
        """Queue one request (the integrals of one request() fan-out); returns its ticket."""
        n = len(integrals)
        arr = integral_array(integrals)
        t = C.c_uint64()
        self.check(capi.lib().gb_submit(self.h, arr, n, _table_array(tables), len(tables), PREC[precision],
                                        C.byref(t)))
        return Ticket(self, int(t.value), n)

    def stats(self) -> dict:
        st = capi.Stats()
        self.check(capi.lib().gb_get_stats(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in capi.Stats._fields_}

    def reset_stats(self):
        self.check(capi.lib().gb_reset_stats(self.h))

    def selftest_wait(self, max_cycles: int = 1 << 20) -> int:
        """Status of gb_selftest_wait: GB_ETIMEDOUT (4) when the bounded wait gave up as designed."""
        return capi.lib().gb_selftest_wait(self.h, max_cycles)

    def measure_peaks(self):
        """(FP32 TFLOP/s, MUFU G op/s, FP64 TFLOP/s) of this GPU from the library's probes."""
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        self.check(capi.lib().gb_measure_peaks(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def close(self):
        if self.h:
            capi.lib().gb_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
