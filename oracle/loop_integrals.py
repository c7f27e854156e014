"""FP64 numpy restatement of DiFfRG's host loop integrals and extent fits -- TEST INFRASTRUCTURE ONLY.

Only ``tests/`` imports this module.  It restates, term by term,
  * DiFfRG/include/DiFfRG/physics/loop_integrals.hh:34-655 (LoopIntegrals::integrate,
    angle_integrate, two_angle_integrate, three_angle_integrate, spatial_integrate_and_integrate,
    spatial_angle_integrate_and_integrate, spatial_integrate_and_sum,
    spatial_angle_integrate_and_sum, sum), vectorised over the tensor-product grid;
  * DiFfRG/src/DiFfRG/physics/flow_equations.cc:54-103 and 161-285 (the x_extent, q0_extent and
    x0_extent fits).
The Gauss rules on [0,1] come from the oracle's own Gauss-Legendre routine (``oracle.gauss_legendre``),
which is pinned to the reference's constexpr tables (tests/golden/gl_tables.json).

Parity pins: the closed forms of the reference's own tests
(DiFfRG/tests/physics/test_loop_integrals.cc:16-289: polynomial integrands, the Riemann-zeta
Matsubara sums) are checked against this restatement in tests/test_loop_integrals.py.

two_angle_integrate: the reference weights its phi nodes with the weight of the current cos node
(loop_integrals.hh:180-181); ``two_angle_integrate(..., reference_phi_weight=True)`` restates that
literally, the default the integral the reference documents (phi weights of the phi rule).
"""
from __future__ import annotations

import math
from functools import lru_cache

import numpy as np

from . import oracle as _orc

PI = math.pi


@lru_cache(maxsize=64)
def _rule(n: int):
    x, w = _orc.gauss_legendre(int(n))
    x.setflags(write=False)
    w.setflags(write=False)
    return x, w


def rule(n: int):
    """n-point Gauss-Legendre rule on [0,1], weights summing to 1."""
    return _rule(int(n))


def sphere_area(d: float) -> float:
    return 2.0 * PI ** (d / 2.0) / math.gamma(d / 2.0)


def _radial(n_x, x_extent, k, d):
    """q^2, weight x measure factor of the x axis: x_w * (0.5 k^d x^((d-2)/2))."""
    xp, xw = rule(n_x)
    x = xp * x_extent
    xwt = xw * x_extent
    q2 = x * k * k
    return q2, xwt * (0.5 * k ** d * np.power(x, (d - 2) / 2.0))


def integrate(f, d, n_x, x_extent, k):
    """loop_integrals.hh:34-66; f(q2) vectorised."""
    q2, wr = _radial(n_x, x_extent, k, d)
    pref = sphere_area(d) * (2 * PI) ** (-d)
    return complex_or_real(np.sum(pref * wr * f(q2)))


def angle_integrate(f, d, n_x, x_extent, k, n_cos):
    """loop_integrals.hh:83-125; f(q2, cos)."""
    q2, wr = _radial(n_x, x_extent, k, d)
    cp, cw = rule(n_cos)
    c = (cp - 0.5) * 2.0
    cwt = cw * 2.0
    pref = sphere_area(d) * (2 * PI) ** (-d)
    Q, C = np.meshgrid(q2, c, indexing="ij")
    W = np.outer(wr, 0.5 * cwt)
    return complex_or_real(np.sum(pref * W * f(Q, C)))


def two_angle_integrate(f, d, n_x, x_extent, k, n_cos, reference_phi_weight=False):
    """loop_integrals.hh:144-194; f(q2, cos, phi), phi nodes of the cos rule on [0, 2 pi]."""
    q2, wr = _radial(n_x, x_extent, k, d)
    cp, cw = rule(n_cos)
    c = (cp - 0.5) * 2.0
    cwt = cw * 2.0
    phi = cp * 2 * PI
    pref = sphere_area(d) * (2 * PI) ** (-d)
    Q, C, P = np.meshgrid(q2, c, phi, indexing="ij")
    if reference_phi_weight:
        pw = np.broadcast_to((cw * 2 * PI)[None, :, None], Q.shape)  # the cos node's weight
    else:
        pw = np.broadcast_to((cw * 2 * PI)[None, None, :], Q.shape)
    W = wr[:, None, None] * (0.5 * cwt)[None, :, None] * pw / (2 * PI)
    return complex_or_real(np.sum(pref * W * f(Q, C, P)))


def three_angle_integrate(f, d, n_x, x_extent, k, n_cos):
    """loop_integrals.hh:214-275; f(q2, cos1, cos2, phi), sqrt(1 - cos1^2) on the first angle."""
    q2, wr = _radial(n_x, x_extent, k, d)
    cp, cw = rule(n_cos)
    c = (cp - 0.5) * 2.0
    c1w = cw * 2.0 * np.sqrt(1.0 - c * c)
    c2w = cw * 2.0
    phi = cp * 2 * PI
    phw = cw * 2 * PI
    pref = sphere_area(d) * (2 * PI) ** (-d)
    S4 = sphere_area(4)
    Q, C1, C2, P = np.meshgrid(q2, c, c, phi, indexing="ij")
    W = (wr[:, None, None, None] * c1w[None, :, None, None] * c2w[None, None, :, None] *
         phw[None, None, None, :] / S4)
    return complex_or_real(np.sum(pref * W * f(Q, C1, C2, P)))


def _spatial_pref(d):
    ds = d - 1
    return ds, sphere_area(ds) * (2 * PI) ** (-ds)


def spatial_integrate_and_integrate(f, d, n_x, x_extent, k, n_m, m_extent):
    """loop_integrals.hh:295-333; f(q2, q0), q0 in [0, m_extent] symmetrised."""
    ds, pref = _spatial_pref(d)
    q2, wr = _radial(n_x, x_extent, k, ds)
    mp, mw = rule(n_m)
    q0 = mp * m_extent
    mwt = mw * m_extent
    Q, Q0 = np.meshgrid(q2, q0, indexing="ij")
    W = np.outer(wr, mwt / (2 * PI))
    return complex_or_real(np.sum(pref * W * (f(Q, Q0) + f(Q, -Q0))))


def spatial_angle_integrate_and_integrate(f, d, n_x, x_extent, k, n_cos, n_m, m_extent):
    """loop_integrals.hh:359-409; f(q2, cos, q0)."""
    ds, pref = _spatial_pref(d)
    q2, wr = _radial(n_x, x_extent, k, ds)
    cp, cw = rule(n_cos)
    c = (cp - 0.5) * 2.0
    mp, mw = rule(n_m)
    q0 = mp * m_extent
    mwt = mw * m_extent
    Q, C, Q0 = np.meshgrid(q2, c, q0, indexing="ij")
    W = wr[:, None, None] * (0.5 * cw * 2.0)[None, :, None] * (mwt / (2 * PI))[None, None, :]
    return complex_or_real(np.sum(pref * W * (f(Q, C, Q0) + f(Q, C, -Q0))))


def _tail(n_m, m_extent, m_order, T):
    """The q0 tail rule of loop_integrals.hh:481-499: nodes and weights / (2 pi)."""
    mp, mw = rule(n_m)
    q0 = (2.0 * m_order * PI * T) + mp * (m_extent - 2.0 * (m_order + 1) * PI * T)
    wt = mw * (m_extent - 2.0 * m_order * PI * T)
    return q0, wt / (2 * PI)


def spatial_integrate_and_sum(f, d, n_x, x_extent, k, m_order, n_m, m_extent, T):
    """loop_integrals.hh:435-504; f(q2, q0)."""
    if abs(T) <= np.finfo(float).eps:
        return spatial_integrate_and_integrate(f, d, n_x, x_extent, k, n_m, m_extent)
    ds, pref = _spatial_pref(d)
    q2, wr = _radial(n_x, x_extent, k, ds)
    n = np.arange(-m_order, m_order + 1)
    Q, Q0 = np.meshgrid(q2, 2.0 * PI * T * n, indexing="ij")
    s = np.sum(pref * T * wr[:, None] * f(Q, Q0))
    q0, tw = _tail(n_m, m_extent, m_order, T)
    Q, Q0 = np.meshgrid(q2, q0, indexing="ij")
    i = np.sum(pref * np.outer(wr, tw) * (f(Q, Q0) + f(Q, -Q0)))
    return complex_or_real(s + i)


def spatial_angle_integrate_and_sum(f, d, n_x, x_extent, k, n_cos, m_order, n_m, m_extent, T):
    """loop_integrals.hh:528-616; f(q2, cos, q0)."""
    if abs(T) <= np.finfo(float).eps:
        return spatial_angle_integrate_and_integrate(f, d, n_x, x_extent, k, n_cos, n_m, m_extent)
    ds, pref = _spatial_pref(d)
    q2, wr = _radial(n_x, x_extent, k, ds)
    cp, cw = rule(n_cos)
    c = (cp - 0.5) * 2.0
    ca = 0.5 * cw * 2.0
    n = np.arange(-m_order, m_order + 1)
    Q, C, Q0 = np.meshgrid(q2, c, 2.0 * PI * T * n, indexing="ij")
    s = np.sum(pref * T * wr[:, None, None] * ca[None, :, None] * f(Q, C, Q0))
    q0, tw = _tail(n_m, m_extent, m_order, T)
    Q, C, Q0 = np.meshgrid(q2, c, q0, indexing="ij")
    W = wr[:, None, None] * ca[None, :, None] * tw[None, None, :]
    i = np.sum(pref * W * (f(Q, C, Q0) + f(Q, C, -Q0)))
    return complex_or_real(s + i)


def loop_sum(f, m_order, n_m, m_extent, T):
    """loop_integrals.hh:618-655 (LoopIntegrals::sum); f(q0)."""
    s = 0.0
    if abs(T) > np.finfo(float).eps:
        n = np.arange(-m_order, m_order + 1)
        s = np.sum(T * f(2.0 * PI * T * n))
    q0, tw = _tail(n_m, m_extent, m_order, T)
    return complex_or_real(s + np.sum(tw * (f(q0) + f(-q0))))


def complex_or_real(v):
    v = complex(v)
    return v if v.imag != 0.0 else v.real


# ---------------------------------------------------------------------------------------------
# extent fits (flow_equations.cc)
# ---------------------------------------------------------------------------------------------
QUADRATURE_FACTOR = 5  # flow_equations.cc:11


class ExtentError(RuntimeError):
    pass


def _fit(integral, order, extent, tol, max_rises):
    """The loop of flow_equations.cc:82-102; returns (extent, number of evaluations)."""
    n1, n2, n3 = QUADRATURE_FACTOR * order, QUADRATURE_FACTOR * 2 * order, QUADRATURE_FACTOR * 10 * order
    eps1 = eps2 = 1.0
    counter = 0
    steps = 0
    while eps1 > tol or eps2 > tol:
        I1 = integral(n1, extent)
        I2 = integral(n2, 2.0 * extent)
        I3 = integral(n3, 10.0 * extent)
        steps += 1
        r1 = abs((I2 - I1) / I1)
        r2 = abs((I2 - I3) / I2)
        counter = counter + 1 if (r1 > eps1 and r2 > eps2) else 0
        if counter > max_rises:
            raise ExtentError("cannot reach the requested precision")
        eps1, eps2 = r1, r2
        if eps1 > tol or eps2 > tol:
            extent *= 1.15
    return extent, steps


def _probe_zero(f):
    for i in range(10):
        x = 1.0 + 1e-3 + (1.5 ** i - 1.0)
        if abs(f(np.array([x]))[0]) > np.finfo(float).eps:
            return False
    return True


def fit_x_extent(optimize_x, x_order, tol, k=1.0):
    """FlowEquations{,FiniteT}::update_x_extent (flow_equations.cc:54-103, 161-206)."""
    if _probe_zero(optimize_x):
        return 1.0, 0
    return _fit(lambda n, ext: integrate(optimize_x, 4, n, ext, k), x_order, 1.0, tol, 2)


def fit_q0_extent(optimize_q0, q0_order, tol, x_extent, k=1.0):
    """FlowEquationsFiniteT::update_q0_extent (flow_equations.cc:208-247)."""
    return _fit(lambda n, ext: abs(loop_sum(optimize_q0, 0, n, ext, 0.0)), q0_order, 0.5 * math.sqrt(x_extent) * k,
                tol, 2)


def fit_x0_extent(optimize_x0, x0_order, tol, x_extent, k=1.0):
    """FlowEquationsFiniteT::update_x0_extent (flow_equations.cc:249-285)."""
    return _fit(lambda n, ext: abs(loop_sum(optimize_x0, 0, n, ext * k, 0.0)), x0_order, 0.5 * math.sqrt(x_extent),
                tol, 1)
