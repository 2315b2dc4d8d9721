"""Oracle restatement of the node-centred Lagrange WENO-5 first derivative on nonuniform
grids, ``src/discretization/schemes/WENO/nonuniform_weno.jl:1-212`` (Fornberg 1988
three-point weights, Jiang-Shu smoothness indicators by Simpson quadrature, Shi-Hu-Shu 2002
positive/negative splitting of the ideal weights, theta = 3), evaluated from the grid
coordinates each time as the reference does.  Python floats are IEEE binary64 without
contraction, like Julia without ``@fastmath``/``muladd``.

Test infrastructure only: imported by tests and the CPU baseline, never by the product.
"""
from __future__ import annotations

import numpy as np


def fornberg3_weights(a, xt):
    """``_fornberg3_weights`` (nonuniform_weno.jl:5-52): the m = 0, 1, 2 weights at xt on the
    three nodes a, in the reference's operation order."""
    a0, a1, a2 = a
    n1m0, n1m1, n1m2 = 1.0, 0.0, 0.0
    c1 = 1.0
    c2 = a1 - a0
    r1 = c1 / c2
    tA = a1 - xt
    a1m0 = (tA * n1m0) / c2
    a1m1 = (tA * n1m1 - n1m0) / c2
    a1m2 = (tA * n1m2 - 2 * n1m1) / c2
    sB = a0 - xt
    a2m0 = r1 * (-(sB) * n1m0)
    a2m1 = r1 * (n1m0 - sB * n1m1)
    a2m2 = r1 * (2 * n1m1 - sB * n1m2)
    c1 = c2
    n1m0, n1m1, n1m2 = a1m0, a1m1, a1m2
    n2m0, n2m1, n2m2 = a2m0, a2m1, a2m2
    c2 = (a2 - a0) * (a2 - a1)
    r2 = c1 / c2
    c3a = a2 - a0
    c3b = a2 - a1
    tA2 = a2 - xt
    b1m0 = (tA2 * n1m0) / c3a
    b1m1 = (tA2 * n1m1 - n1m0) / c3a
    b1m2 = (tA2 * n1m2 - 2 * n1m1) / c3a
    b2m0 = (tA2 * n2m0) / c3b
    b2m1 = (tA2 * n2m1 - n2m0) / c3b
    b2m2 = (tA2 * n2m2 - 2 * n2m1) / c3b
    sB2 = a1 - xt
    b3m0 = r2 * (-(sB2) * n2m0)
    b3m1 = r2 * (n2m0 - sB2 * n2m1)
    b3m2 = r2 * (2 * n2m1 - sB2 * n2m2)
    return (b1m0, b2m0, b3m0), (b1m1, b2m1, b3m1), (b1m2, b2m2, b3m2)


def _dot3(w, a, b, c):
    return w[0] * a + w[1] * b + w[2] * c


def _substencil_beta_r(al, ua, ub, uc, xi, xL, xM, xph, dx):
    _, m1i, _ = fornberg3_weights(al, xi)
    _, m1L, _ = fornberg3_weights(al, xL)
    _, m1M, m2M = fornberg3_weights(al, xM)
    _, m1R, _ = fornberg3_weights(al, xph)
    r = _dot3(m1i, ua, ub, uc)
    pL = _dot3(m1L, ua, ub, uc)
    pM = _dot3(m1M, ua, ub, uc)
    pR = _dot3(m1R, ua, ub, uc)
    pp = _dot3(m2M, ua, ub, uc)
    I1 = (dx / 6) * (pL * pL + 4 * (pM * pM) + pR * pR)
    I2 = dx * (pp * pp)
    val = dx * I1 + (dx * dx * dx) * I2
    return np.maximum(val, 0.0), r


def target_geometry(tg, x1, x2, x3, x4, x5):
    """``_weno_target_geometry`` (nonuniform_weno.jl:77-83): (xi, xL, xph)."""
    if tg == 1:
        return x1, x1, (x1 + x2) / 2
    if tg == 2:
        return x2, (x1 + x2) / 2, (x2 + x3) / 2
    if tg == 3:
        return x3, (x2 + x3) / 2, (x3 + x4) / 2
    if tg == 4:
        return x4, (x3 + x4) / 2, (x4 + x5) / 2
    return x5, (x4 + x5) / 2, x5


def ideal_d0d2(tg, x1, x2, x3, x4, x5):
    """``_weno_ideal_d0d2`` (nonuniform_weno.jl:86-117)."""
    if tg == 3:
        d0 = ((x3 - x4) * (x3 - x5)) / ((x1 - x4) * (x1 - x5))
        d2 = ((x3 - x1) * (x3 - x2)) / ((x5 - x1) * (x5 - x2))
    elif tg == 1:
        d0 = (((2 * x1 - x2 - x3) * (x1 - x4) * (x1 - x5) + (x1 - x3) * (x1 - x5) * (x1 - x2)
               + (x1 - x3) * (x1 - x4) * (x1 - x2)) / ((2 * x1 - x2 - x3) * (x1 - x4) * (x1 - x5)))
        d2 = ((x1 - x3) * (x1 - x4) * (x1 - x2)) / ((-x1 + x5) * (2 * x1 - x3 - x4) * (-x2 + x5))
    elif tg == 2:
        d0 = ((x2 - x4) * (x2 - x5)) / ((x1 - x4) * (x1 - x5))
        d2 = ((-x1 + x2) * (x2 - x3) * (x2 - x4)) / ((-x1 + x5) * (2 * x2 - x3 - x4) * (-x2 + x5))
    elif tg == 4:
        d0 = ((-x2 + x4) * (-x3 + x4) * (x4 - x5)) / ((x1 - x4) * (x1 - x5) * (-x2 - x3 + 2 * x4))
        d2 = ((-x1 + x4) * (-x2 + x4)) / ((-x1 + x5) * (-x2 + x5))
    else:
        d0 = ((-x2 + x5) * (-x3 + x5) * (-x4 + x5)) / ((x1 - x4) * (x1 - x5) * (-x2 - x3 + 2 * x5))
        d2 = (((-x1 - x4 + 2 * x5) * (-x2 + x5) * (-x3 + x5) + (-x1 + x5) * (-x2 - x3 + 2 * x5) * (-x4 + x5))
              / ((-x1 + x5) * (-x2 + x5) * (-x3 - x4 + 2 * x5)))
    return d0, d2


def weno_f_nonuniform(u, eps, x, tg=3):
    """``_weno_f_nonuniform_core`` (nonuniform_weno.jl:120-163) for the five values u at the
    five nodes x, target node tg (1..5)."""
    theta = 3.0
    half = 1.0 / 2
    x1, x2, x3, x4, x5 = (float(v) for v in x)
    u1, u2, u3, u4, u5 = u
    xi, xL, xph = target_geometry(tg, x1, x2, x3, x4, x5)
    dx = xph - xL
    xM = (xL + xph) / 2
    b0, r0 = _substencil_beta_r((x1, x2, x3), u1, u2, u3, xi, xL, xM, xph, dx)
    b1, r1 = _substencil_beta_r((x2, x3, x4), u2, u3, u4, xi, xL, xM, xph, dx)
    b2, r2 = _substencil_beta_r((x3, x4, x5), u3, u4, u5, xi, xL, xM, xph, dx)
    d0, d2 = ideal_d0d2(tg, x1, x2, x3, x4, x5)
    d1 = 1.0 - d0 - d2
    dp0 = half * (d0 + theta * abs(d0))
    dp1 = half * (d1 + theta * abs(d1))
    dp2 = half * (d2 + theta * abs(d2))
    dm0, dm1, dm2 = dp0 - d0, dp1 - d1, dp2 - d2
    sp_ = dp0 + dp1 + dp2
    sm_ = dm0 + dm1 + dm2
    ap0 = (dp0 / sp_) / ((eps + b0) * (eps + b0))
    ap1 = (dp1 / sp_) / ((eps + b1) * (eps + b1))
    ap2 = (dp2 / sp_) / ((eps + b2) * (eps + b2))
    s_p = ap0 + ap1 + ap2
    am0 = (dm0 / sm_) / ((eps + b0) * (eps + b0))
    am1 = (dm1 / sm_) / ((eps + b1) * (eps + b1))
    am2 = (dm2 / sm_) / ((eps + b2) * (eps + b2))
    s_m = am0 + am1 + am2
    Rp = (ap0 / s_p) * r0 + (ap1 / s_p) * r1 + (ap2 / s_p) * r2
    Rm = (am0 / s_m) * r0 + (am1 / s_m) * r1 + (am2 / s_m) * r2
    return sp_ * Rp - sm_ * Rm


def taps_and_target(i: int, n: int):
    """``get_f_taps_coords`` without interfaces (function_scheme.jl:1-34) for the WENO scheme's
    two lower and two upper boundary functions (WENO.jl:84-85): (1-based taps, target)."""
    if i <= 2:
        return list(range(1, 6)), i
    if i > n - 2:
        return list(range(n - 4, n + 1)), 5 - (n - i)
    return list(range(i - 2, i + 3)), 3
