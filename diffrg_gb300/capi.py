"""ctypes binding of libgbint.so (the C ABI declared in include/gbint.h).

This is the Python host side above the C ABI: the same entry points a C++ or Fortran host
binds.  The library must be the in-tree build (diffrg_gb300/lib/libgbint.so); there is no
fallback -- a missing library or a missing GPU raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libgbint.so")

GB_OK, GB_EINVAL, GB_ENOMEM, GB_EBUDGET, GB_ETIMEDOUT, GB_ECUDA, GB_ENODEV, GB_EAGAIN, GB_EDEVICE, GB_ECANCELED = range(10)

FAM = {
    "1D": 1, "ANGLE": 2, "3D": 3, "4D2ANG": 4, "4D": 5, "CART1": 6, "CART2": 7, "CART3": 8,
    "2DPQ0": 9, "2DPX0": 10, "3DPQ0": 11, "3DPX0": 12, "FTQ0": 13, "ANGLE_FTQ0": 14, "4D_FTQ0": 15,
    "FTX0": 16, "ANGLE_FTX0": 17, "4D_FTX0": 18, "CONST": 19, "QLOOP": 20, "QLOOP_T": 21,
}
IG = {"POLY": 0, "PROP1": 1, "PROP3": 3, "VERT4": 5, "FTLOOP": 6}
PREC = {"fp32c": 0, "fp64": 1, "fp32f": 2, "fp32a": 3}
GB_MAX_ARGS = 24

# C ABI symbols declared in include/gbint.h (checked by the CPU test suite)
EXPORTS = [
    "gb_version", "gb_status_string", "gb_ctx_create", "gb_ctx_destroy", "gb_last_error",
    "gb_quad_gl", "gb_quad_rule", "gb_quad_rule_host", "gb_quad_matsubara", "gb_quad_config",
    "gb_table_create", "gb_table_update", "gb_table_update_device", "gb_table_update_many", "gb_table_epoch",
    "gb_table_destroy",
    "gb_batch_create", "gb_batch_run", "gb_batch_run_graph", "gb_batch_results", "gb_batch_get",
    "gb_batch_run_plain", "gb_batch_info", "gb_batch_destroy", "gb_get", "gb_get_noalloc",
    "gb_serve_start", "gb_serve_start_device", "gb_serve_device_info", "gb_serve_stop", "gb_submit", "gb_poll", "gb_wait", "gb_cancel",
    "gb_get_stats", "gb_reset_stats", "gb_measure_peaks",
    "gb_buffer_create", "gb_buffer_upload", "gb_buffer_destroy",
    "gb_slot_acquire", "gb_slot_wait", "gb_slot_release", "gb_slot_host", "gb_device_info",
    "gb_graph_capture_begin", "gb_graph_capture_end", "gb_graph_launch", "gb_graph_info", "gb_graph_destroy",
    "gb_autotune", "gb_tune_set", "gb_tune_set_schedule", "gb_tune_get_schedule", "gb_tune_report", "gb_selftest_wait", "gb_table_group_begin", "gb_table_group_end",
]


class TableSpec(C.Structure):
    _fields_ = [("n0", C.c_int), ("log0", C.c_int), ("lo0", C.c_double), ("hi0", C.c_double),
                ("n1", C.c_int), ("log1", C.c_int), ("lo1", C.c_double), ("hi1", C.c_double)]


class Integral(C.Structure):
    _fields_ = [("family", C.c_int), ("integrand", C.c_int), ("d", C.c_int), ("n", C.c_int * 4), ("table_base", C.c_int),
                ("x_extent", C.c_double), ("x0_extent", C.c_double), ("x0_summands", C.c_int),
                ("T", C.c_double), ("E", C.c_double), ("k", C.c_double),
                ("qmin", C.c_double * 3), ("qmax", C.c_double * 3), ("args", C.c_double * GB_MAX_ARGS)]


class Schedule(C.Structure):
    _fields_ = [("threads", C.c_int), ("rows_per_thread", C.c_int), ("inner_split", C.c_int), ("unit_order", C.c_int)]


GB_ORDER_ITEM, GB_ORDER_COST = 0, 1


class Stats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("batches_launched", C.c_uint64), ("points_evaluated", C.c_uint64),
                ("busy_seconds", C.c_double), ("p50_latency_s", C.c_double), ("p99_latency_s", C.c_double),
                ("max_latency_s", C.c_double), ("bytes_in_use", C.c_uint64), ("bytes_budget", C.c_uint64)]


_lib = None


class GbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_status(code), code, msg))
        self.code = code


def _status(code):
    try:
        return lib().gb_status_string(code).decode()
    except Exception:
        return "status"


def load(path: str = LIB_PATH):
    """Load the in-tree library (build it first with diffrg_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libgbint.so not built: run `python -c 'import __graft_entry__ as g; g.build()'`")
    L = C.CDLL(path)
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    L.gb_version.restype = C.c_int
    L.gb_status_string.restype = C.c_char_p
    L.gb_status_string.argtypes = [C.c_int]
    L.gb_ctx_create.argtypes = [C.c_int, C.c_size_t, C.POINTER(vp)]
    L.gb_ctx_destroy.argtypes = [vp]
    L.gb_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.gb_quad_gl.argtypes = [vp, C.c_int, C.c_int, C.POINTER(dp), C.POINTER(dp), C.POINTER(vp), C.POINTER(vp)]
    L.gb_quad_rule.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(dp), C.POINTER(dp), C.POINTER(vp),
                               C.POINTER(vp)]
    L.gb_quad_rule_host.argtypes = [C.c_int, C.c_int, dp, dp]
    L.gb_quad_matsubara.argtypes = [vp, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_int), C.POINTER(dp),
                                    C.POINTER(dp), C.POINTER(vp), C.POINTER(vp), dp]
    L.gb_quad_config.argtypes = [vp, C.c_int, C.c_int, C.c_int]
    L.gb_table_create.argtypes = [vp, C.POINTER(TableSpec), C.POINTER(vp)]
    L.gb_table_update.argtypes = [vp, vp, C.POINTER(C.c_float), vp]
    L.gb_table_update_device.argtypes = [vp, vp, vp, vp]
    L.gb_table_update_many.argtypes = [vp, C.c_int, vp, vp, vp]
    L.gb_table_epoch.argtypes = [vp, vp, C.POINTER(C.c_uint64)]
    L.gb_table_destroy.argtypes = [vp, vp]
    L.gb_batch_create.argtypes = [vp, C.POINTER(Integral), C.c_int, C.POINTER(vp), C.c_int, C.c_int, C.POINTER(vp)]
    L.gb_batch_run.argtypes = [vp, vp, vp, vp]
    L.gb_batch_run_graph.argtypes = [vp, vp, vp]
    L.gb_batch_results.argtypes = [vp, vp, dp, vp]
    L.gb_batch_get.argtypes = [vp, vp, dp, vp]
    L.gb_batch_run_plain.argtypes = [vp, vp, dp, C.c_int]
    L.gb_batch_info.argtypes = [vp, vp, C.POINTER(C.c_uint64), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.gb_batch_destroy.argtypes = [vp, vp]
    L.gb_get.argtypes = [vp, C.POINTER(Integral), C.POINTER(vp), C.c_int, C.c_int, dp]
    L.gb_get_noalloc.argtypes = [vp, C.POINTER(Integral), C.POINTER(vp), C.c_int, dp]
    L.gb_serve_start.argtypes = [vp, C.c_int, C.c_int]
    L.gb_serve_stop.argtypes = [vp]
    L.gb_serve_start_device.argtypes = [vp, C.c_int, C.c_int, C.c_longlong, C.c_double]
    L.gb_serve_device_info.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.gb_submit.argtypes = [vp, C.POINTER(Integral), C.c_int, C.POINTER(vp), C.c_int, C.c_int,
                            C.POINTER(C.c_uint64)]
    L.gb_poll.argtypes = [vp, C.c_uint64, dp]
    L.gb_wait.argtypes = [vp, C.c_uint64, dp, C.c_double]
    L.gb_cancel.argtypes = [vp, C.c_uint64]
    L.gb_get_stats.argtypes = [vp, C.POINTER(Stats)]
    L.gb_reset_stats.argtypes = [vp]
    L.gb_measure_peaks.argtypes = [vp, dp, dp, dp]
    L.gb_graph_capture_begin.argtypes = [vp, vp]
    L.gb_graph_capture_end.argtypes = [vp, vp, C.POINTER(vp)]
    L.gb_graph_launch.argtypes = [vp, vp, vp]
    L.gb_graph_info.argtypes = [vp, vp, C.POINTER(C.c_int)]
    L.gb_graph_destroy.argtypes = [vp, vp]
    L.gb_tune_set_schedule.argtypes = [vp, C.c_int, C.POINTER(Schedule)]
    L.gb_tune_get_schedule.argtypes = [vp, C.c_int, C.POINTER(Schedule)]
    L.gb_tune_report.argtypes = [vp, C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]
    L.gb_autotune.argtypes = [vp, C.POINTER(Integral), C.c_int, C.POINTER(vp), C.c_int, C.c_int, C.c_char_p, C.c_int,
                              C.POINTER(C.c_int)]
    L.gb_tune_set.argtypes = [vp, C.c_int, C.c_int]
    L.gb_selftest_wait.argtypes = [vp, C.c_longlong]
    L.gb_device_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.gb_table_group_begin.argtypes = [vp]
    L.gb_table_group_end.argtypes = [vp]
    _lib = L
    return L


def lib():
    return load()


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))
