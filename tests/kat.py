"""Known-answer integrals of the polynomial test KERNEL for every integrator family.

Restates, as closed forms, the analytic references of the reference's integrator tests
(DiFfRG/tests/physics/integration/integrator_*_{cpu,gpu}.{cc,cu} and
DiFfRG/tests/physics/integration_finiteT/*.{cc,cu}): volume integrals V_d/(2 pi)^d and random
polynomial integrals built from Polynomial::integral.
"""
import math

import numpy as np

P = np.polynomial.polynomial
TP = 2 * math.pi


def S_d(d):
    return 2 * math.pi ** (d / 2) / math.gamma(d / 2)


def pint(c, a, b, shift=0):
    """int_a^b (sum_i c_i x^i) x^shift dx"""
    c = np.concatenate([np.zeros(shift), np.asarray(c, dtype=float)])
    ci = P.polyint(c)
    return P.polyval(b, ci) - P.polyval(a, ci)


def sqrt_moment(c):
    """int_-1^1 sqrt(1-c^2) P(c) dc for a cubic P"""
    return c[0] * math.pi / 2 + c[2] * math.pi / 8


def random_args(rng, q0_rational=None):
    """Coefficients like the reference's GENERATE(random(-1,1)); q0_rational=(T, v) gives the
    finite-T kernel factor 1/(T^2 + v^2 q0^2)."""
    a = np.zeros(24)
    a[0] = rng.uniform(-1, 1)
    a[1:7] = rng.uniform(-1, 1, 6)
    a[7:11] = rng.uniform(-1, 1, 4)
    a[11:15] = rng.uniform(-1, 1, 4)
    a[15:19] = rng.uniform(-1, 1, 4)
    a[19:23] = rng.uniform(-1, 1, 4)
    if q0_rational is not None:
        T, v = q0_rational
        a[19:23] = [T * T, 0.0, v * v, 0.0]
        a[23] = 1.0
    return a


def analytic(family, a, k, d=4, x_extent=1.0, x0_extent=0.0, x0_summands=0, T=0.0, qmin=(-math.pi,) * 3,
             qmax=(math.pi,) * 3):
    c = a[0]
    pq, p1, p2, p3, pt = a[1:7], a[7:11], a[11:15], a[15:19], a[19:23]
    qe = math.sqrt(x_extent) * k
    cosI = pint(p1, -1, 1)
    if family == "1D":
        return c + S_d(d) * pint(pq, 0, qe, d - 1) / TP ** d
    if family == "ANGLE":
        return c + S_d(d) * pint(pq, 0, qe, d - 1) * 0.5 * cosI / TP ** d
    if family == "3D":
        return c + pint(pq, 0, qe, 2) * cosI * pint(p2, 0, TP) / TP ** 3
    if family == "4D2ANG":
        return c + TP * pint(pq, 0, qe, 3) * sqrt_moment(p1) * pint(p2, -1, 1) / TP ** 4
    if family == "4D":
        return c + pint(pq, 0, qe, 3) * sqrt_moment(p1) * pint(p2, -1, 1) * pint(p3, 0, TP) / TP ** 4
    if family.startswith("CART"):
        dim = int(family[-1])
        v = pint(pq, qmin[0], qmax[0])
        if dim > 1:
            v *= pint(p1, qmin[1], qmax[1])
        if dim > 2:
            v *= pint(p2, qmin[2], qmax[2])
        return c + v / TP ** dim
    if family in ("2DPQ0", "2DPX0"):
        L = x0_extent * (k if family == "2DPX0" else 1.0)
        return c + S_d(2) / 2 * pint(pq, 0, qe, 1) * cosI * pint(pt, -L, L) / TP ** 3
    if family in ("3DPQ0", "3DPX0"):
        L = x0_extent * (k if family == "3DPX0" else 1.0)
        return c + pint(pq, 0, qe, 2) * cosI * pint(p2, 0, TP) * pint(pt, -L, L) / TP ** 4
    if family in ("FTQ0", "ANGLE_FTQ0", "4D_FTQ0"):
        # kernel q0 factor 1/(T^2 + v^2 q0^2) -> T sum_n = 1/(2 v T tanh(1/(2v)))
        v = math.sqrt(a[21])
        msum = 1.0 / (2 * v * T * math.tanh(1 / (2 * v)))
        if family == "4D_FTQ0":
            spatial = pint(pq, 0, qe, 2) * cosI * pint(p2, 0, TP) / TP ** 3
        else:
            dd = d
            spatial = S_d(dd - 1) * pint(pq, 0, qe, dd - 2) / TP ** (dd - 1)
            if family == "ANGLE_FTQ0":
                spatial *= 0.5 * cosI
        return c + spatial * msum
    if family in ("FTX0", "ANGLE_FTX0", "4D_FTX0"):
        Tzero = abs(T) < 1e-12
        ns = 0 if Tzero else x0_summands
        ssum = 0.0
        for m in range(ns):
            q0 = TP * T * m
            ssum += T * (P.polyval(0.0, pt) if m == 0 else P.polyval(q0, pt) + P.polyval(-q0, pt))
        lo = TP * T * ns
        hi = k * x0_extent if not Tzero else k * (x0_extent - 1e-3)
        even = np.array(pt, dtype=float) * np.array([2, 0, 2, 0])
        tail = pint(even, lo, hi) / TP
        if family == "4D_FTX0":
            spatial = pint(pq, 0, qe, 2) * cosI * pint(p2, 0, TP) / TP ** 3
        else:
            spatial = S_d(d - 1) * pint(pq, 0, qe, d - 2) / TP ** (d - 1)
            if family == "ANGLE_FTX0":
                spatial *= 0.5 * cosI
        return c + spatial * (ssum + tail)
    if family == "CONST":
        return c + P.polyval(k, pq) * S_d(d) / TP ** d
    raise ValueError(family)


# family -> (grid sizes, extra keyword arguments) used by the CPU and GPU known-answer tests
CASES = {
    "1D": dict(n=(64,), d=4),
    "ANGLE": dict(n=(64, 12), d=4),
    "3D": dict(n=(64, 12, 16), d=3),
    "4D2ANG": dict(n=(64, 12, 12), d=4),
    "4D": dict(n=(64, 16, 12, 8), d=4),
    "CART1": dict(n=(16,), d=1, qmin=(-1.0, -0.5, -2.0), qmax=(1.5, 0.5, 1.0)),
    "CART2": dict(n=(16, 12), d=2, qmin=(-1.0, -0.5, -2.0), qmax=(1.5, 0.5, 1.0)),
    "CART3": dict(n=(16, 12, 8), d=3, qmin=(-1.0, -0.5, -2.0), qmax=(1.5, 0.5, 1.0)),
    "2DPQ0": dict(n=(64, 12, 12), d=3, x0_extent=1.3),
    "2DPX0": dict(n=(64, 12, 12), d=3, x0_extent=1.3),
    "3DPQ0": dict(n=(64, 12, 16, 12), d=4, x0_extent=1.3),
    "3DPX0": dict(n=(64, 12, 16, 12), d=4, x0_extent=1.3),
    "FTQ0": dict(n=(64,), d=4, T=0.2),
    "ANGLE_FTQ0": dict(n=(64, 12), d=4, T=0.2),
    "4D_FTQ0": dict(n=(64, 16, 16), d=4, T=0.2),
    "FTX0": dict(n=(64, 64), d=4, T=0.2, x0_summands=32),
    "ANGLE_FTX0": dict(n=(64, 12, 64), d=4, T=0.2, x0_summands=32),
    "4D_FTX0": dict(n=(32, 12, 12, 48), d=4, T=0.2, x0_summands=16),
    "CONST": dict(n=(1,), d=4),
}
