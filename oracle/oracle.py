"""ctypes wrapper of the FP64 CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle is a plain C++ FP64 restatement of DiFfRG's CPU integrators (the
``*_cpu.hh`` TBB twins), its Gauss-Legendre / Golub-Welsch / Monien-Matsubara
quadrature and the benchmark integrands.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import this
module; the product (``diffrg_gb300``) never does.

Parity pins (DiFfRG project paths):
  * GL nodes: DiFfRG/include/DiFfRG/common/quadrature/gauss_legendre.hh tables
    (``tests/golden/gl_tables.json``) and numpy's ``leggauss``.
  * Matsubara sums: closed forms of DiFfRG/tests/common/quadrature/test_matsubara.cc:9-60.
  * Integrator families: analytic polynomial integrals as in
    DiFfRG/tests/physics/integration/*.cc and integration_finiteT/*.cc.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

N_ARGS = 24

FAMILIES = {
    "1D": 1, "ANGLE": 2, "3D": 3, "4D2ANG": 4, "4D": 5, "CART1": 6, "CART2": 7, "CART3": 8,
    "2DPQ0": 9, "2DPX0": 10, "3DPQ0": 11, "3DPX0": 12, "FTQ0": 13, "ANGLE_FTQ0": 14,
    "4D_FTQ0": 15, "FTX0": 16, "ANGLE_FTX0": 17, "4D_FTX0": 18, "CONST": 19,
}
INTEGRANDS = {"POLY": 0, "PROP1": 1, "PROP3": 3, "VERT4": 5}


class OrcTable(C.Structure):
    _fields_ = [("n0", C.c_int), ("log0", C.c_int), ("lo0", C.c_double), ("hi0", C.c_double),
                ("n1", C.c_int), ("log1", C.c_int), ("lo1", C.c_double), ("hi1", C.c_double),
                ("data", C.POINTER(C.c_float))]


class OrcFamilyDesc(C.Structure):
    _fields_ = [("family", C.c_int), ("d", C.c_int), ("n", C.c_int * 4),
                ("x_extent", C.c_double), ("x0_extent", C.c_double), ("x0_summands", C.c_int),
                ("T", C.c_double), ("E", C.c_double),
                ("mats_min", C.c_int), ("mats_vacuum", C.c_int), ("mats_add", C.c_int),
                ("qmin", C.c_double * 3), ("qmax", C.c_double * 3)]


_lib = None


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (g++ -fopenmp); returns the library path."""
    out = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.orc_gauss_legendre.argtypes = [C.c_int, dp, dp]
        L.orc_golub_welsch.argtypes = [C.c_int, dp, dp, C.c_double, dp, dp]
        L.orc_matsubara.argtypes = [C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    dp, dp, C.c_int, dp]
        L.orc_family.argtypes = [C.POINTER(OrcFamilyDesc), C.c_int, C.c_int, dp, dp, C.POINTER(OrcTable),
                                 C.c_int, dp, C.c_int]
        L.orc_w1.argtypes = [C.c_int, ip, ip, dp, dp, C.POINTER(OrcTable), dp, C.c_int]
        L.orc_w2.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, dp, dp, dp, C.POINTER(OrcTable),
                             dp, C.c_int]
        L.orc_table_eval.argtypes = [C.POINTER(OrcTable), C.c_int, dp, dp, dp]
        L.orc_regulator.argtypes = [C.c_int, dp, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def gauss_legendre(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    if lib().orc_gauss_legendre(n, _dp(x), _dp(w)) != 0:
        raise ValueError("bad order")
    return x, w


def golub_welsch(a, b, mu0):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    n = a.size
    x = np.zeros(n)
    w = np.zeros(n)
    if lib().orc_golub_welsch(n, _dp(a), _dp(b), float(mu0), _dp(x), _dp(w)) != 0:
        raise RuntimeError("golub_welsch failed")
    return x, w


def matsubara(T, E=1.0, step=2, min_size=0, max_size=1024, vacuum=48, precision_factor=1):
    """Monien rule as MatsubaraQuadrature(T, E, step, min, max, vacuum, prec); returns (x, w, T_used)."""
    cap = 4096
    x = np.zeros(cap)
    w = np.zeros(cap)
    tu = np.zeros(1)
    n = lib().orc_matsubara(float(T), float(E), step, min_size, max_size, vacuum, precision_factor,
                            _dp(x), _dp(w), cap, _dp(tu))
    if n < 0:
        raise RuntimeError("matsubara failed")
    return x[:n].copy(), w[:n].copy(), float(tu[0])


def matsubara_sum(f, T, E=1.0, **kw):
    """T f(0) + sum_i w_i (f(x_i) + f(-x_i)) -- MatsubaraQuadrature::sum (matsubara.hh)."""
    x, w, tu = matsubara(T, E, **kw)
    return tu * f(0.0) + np.sum(w * (f(x) + f(-x)))


def make_table(spec: dict, data: np.ndarray):
    """spec: {'n0','log0','lo0','hi0', optional 'n1','log1','lo1','hi1'}; data float32 row-major."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    t = OrcTable(spec["n0"], int(spec["log0"]), spec["lo0"], spec["hi0"],
                 spec.get("n1", 0), int(spec.get("log1", 0)), spec.get("lo1", 0.0), spec.get("hi1", 1.0),
                 data.ctypes.data_as(C.POINTER(C.c_float)))
    t._keep = data
    return t


def _tables(tables):
    n = len(tables)
    arr = (OrcTable * max(n, 1))()
    keep = []
    for i, (spec, data) in enumerate(tables):
        t = make_table(spec, data)
        keep.append(t._keep)
        arr[i] = t
    return arr, n, keep


def family_desc(family, d=4, n=(0, 0, 0, 0), x_extent=1.0, x0_extent=0.0, x0_summands=0, T=0.0, E=0.0,
                mats_min=32, mats_vacuum=48, mats_add=0, qmin=(-np.pi,) * 3, qmax=(np.pi,) * 3):
    fam = FAMILIES[family] if isinstance(family, str) else int(family)
    nn = list(n) + [0] * (4 - len(n))
    return OrcFamilyDesc(fam, d, (C.c_int * 4)(*nn), x_extent, x0_extent, x0_summands, T, E,
                         mats_min, mats_vacuum, mats_add, (C.c_double * 3)(*qmin), (C.c_double * 3)(*qmax))


def resolve_E(T, k, E_manual=0.0):
    """Typical energy that a freshly built Integrator*FiniteTq0 uses on its first get(k):
    set_T(T) picks E = 10 T (integrator_finiteTq0_cpu.hh:52-55); get() re-selects E = k when
    |k - E| / max(k, E) > 2.5e-2 (:82-85) unless E was set by hand."""
    if E_manual and E_manual > 0:
        return float(E_manual)
    E = 10.0 * T
    if abs(k - E) / max(k, E) > 2.5e-2:
        E = k
    return float(E)


def family(descs, integrand, k, args, tables=(), threads=0):
    """Evaluate integrals: descs (list of OrcFamilyDesc or one), k (n,), args (n, 24)."""
    args = np.ascontiguousarray(np.atleast_2d(args), dtype=np.float64)
    n = args.shape[0]
    if isinstance(descs, OrcFamilyDesc):
        descs = [descs] * n
    darr = (OrcFamilyDesc * n)(*descs)
    k = np.ascontiguousarray(np.broadcast_to(np.asarray(k, dtype=np.float64), (n,)))
    tarr, nt, keep = _tables(tables)
    out = np.zeros(n)
    ig = INTEGRANDS[integrand] if isinstance(integrand, str) else int(integrand)
    rc = lib().orc_family(darr, ig, n, _dp(k), _dp(args), tarr, nt, _dp(out), threads)
    if rc != 0:
        raise RuntimeError("oracle family evaluation failed")
    return out


def w1(z_table, nq, nc, qmax, p, threads=0):
    p = np.ascontiguousarray(np.atleast_1d(p), dtype=np.float64)
    n = p.size
    nq = np.ascontiguousarray(np.broadcast_to(np.asarray(nq, dtype=np.int32), (n,)))
    nc = np.ascontiguousarray(np.broadcast_to(np.asarray(nc, dtype=np.int32), (n,)))
    qm = np.ascontiguousarray(np.broadcast_to(np.asarray(qmax, dtype=np.float64), (n,)))
    tarr, nt, keep = _tables([z_table])
    out = np.zeros(n)
    if lib().orc_w1(n, _ip(nq), _ip(nc), _dp(qm), _dp(p), tarr, _dp(out), threads) != 0:
        raise RuntimeError("oracle w1 failed")
    return out


def w2(z_table, M, nq, nc, qmax, p, T, Omega=0.0, threads=0):
    p = np.ascontiguousarray(np.atleast_1d(p), dtype=np.float64)
    T = np.ascontiguousarray(np.broadcast_to(np.asarray(T, dtype=np.float64), p.shape))
    Om = np.ascontiguousarray(np.broadcast_to(np.asarray(Omega, dtype=np.float64), p.shape))
    tarr, nt, keep = _tables([z_table])
    out = np.zeros(p.size)
    if lib().orc_w2(p.size, M, nq, nc, float(qmax), _dp(p), _dp(T), _dp(Om), tarr, _dp(out), threads) != 0:
        raise RuntimeError("oracle w2 failed")
    return out


def table_eval(spec, data, x0, x1=None):
    t = make_table(spec, data)
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    out = np.zeros(x0.size)
    if x1 is not None:
        x1 = np.ascontiguousarray(x1, dtype=np.float64)
        lib().orc_table_eval(C.byref(t), x0.size, _dp(x0), _dp(x1), _dp(out))
    else:
        lib().orc_table_eval(C.byref(t), x0.size, _dp(x0), None, _dp(out))
    return out


def regulator(q2):
    q2 = np.ascontiguousarray(q2, dtype=np.float64)
    rb = np.zeros_like(q2)
    rd = np.zeros_like(q2)
    lib().orc_regulator(q2.size, _dp(q2), _dp(rb), _dp(rd))
    return rb, rd
