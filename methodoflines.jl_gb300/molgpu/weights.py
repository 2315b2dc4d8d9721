"""Finite-difference weight tables of the discretisation front end.

The reference computes every table with Fornberg's algorithm
(``src/discretization/schemes/fornberg_calculate_weights.jl:20-65``) and the
DerivativeOperator constructors (``centered_diff_weights.jl:4-75``,
``upwind_diff_weights.jl:4-91``, ``half_offset_weights.jl:4-70``).  The same
Float64 operations, in the same order, are performed here, so the tables are
bit-identical to the reference's; the GPU kernels receive them in the
descriptor's weight pool.
"""
from __future__ import annotations

from dataclasses import dataclass
from fractions import Fraction
from typing import Optional, List, Sequence, Tuple


def fornberg(m: int, z: float, nodes: Sequence[float]) -> List[float]:
    """Weights of the m-th derivative at z on `nodes`, sum-to-zero corrected (m > 0)."""
    n = len(nodes)
    if not m < n:
        raise ValueError("Not enough points for the requested order.")
    xs = [float(v) for v in nodes]
    z = float(z)
    tab = [[0.0] * (m + 1) for _ in range(n)]
    tab[0][0] = 1.0
    c1 = 1.0
    c4 = xs[0] - z
    for i in range(1, n):
        top = min(i, m)
        c2 = 1.0
        c5 = c4
        c4 = xs[i] - z
        row_prev = tab[i - 1]
        for j in range(i):
            c3 = xs[i] - xs[j]
            c2 *= c3
            if j == i - 1:
                row = tab[i]
                for s in range(top, 0, -1):
                    row[s] = c1 * (s * row_prev[s - 1] - c5 * row_prev[s]) / c2
                row[0] = -c1 * c5 * row_prev[0] / c2
            rj = tab[j]
            for s in range(top, 0, -1):
                rj[s] = (c4 * rj[s] - s * rj[s - 1]) / c3
            rj[0] = c4 * rj[0] / c3
        c1 = c2
    w = [r[m] for r in tab]
    if m != 0:
        total = w[0]
        for v in w[1:]:
            total = total + v       # Julia's sum of a short vector: left fold
        w[n // 2] -= total
    return w


def julia_pow(x: float, d: int) -> float:
    """``x^d`` for a runtime Int exponent as Julia evaluates it for d <= 3 (else correctly rounded)."""
    if d == 0:
        return 1.0
    if d == 1:
        return x
    if d == 2:
        return x * x
    if d == 3:
        return x * x * x
    return float(Fraction(x) ** d)


@dataclass
class Operator:
    """A DerivativeOperator in the descriptor's form (see ``mol_op1d``)."""
    L: int
    omin: int
    interior: List[float]
    low: List[List[float]]
    high: List[List[float]]
    bLlo: int
    bLhi: int
    hi_base: int = 0
    # nonuniform grids: one interior row per interior position (rows[k] at position nlo+1+k);
    # `interior` is then rows[0]
    rows: Optional[List[List[float]]] = None

    @property
    def nlo(self):
        return len(self.low)

    @property
    def nhi(self):
        return len(self.high)


def centered(d: int, p: int, dx: float) -> Operator:
    """``CompleteCenteredDifference(d, p, dx)`` (centered_difference/centered_diff_weights.jl:4-75)."""
    if p <= 1:
        raise ValueError("approximation_order must be greater than 1.")    # centered_diff_weights.jl:8
    L = d + p - 1 + (d + p) % 2
    bl = d + p
    h = L // 2
    s = 1.0 / julia_pow(dx, d)
    inner = [s * w for w in fornberg(d, 0.0, range(-h, h + 1))]
    low = [[s * w for w in fornberg(d, float(x0), range(bl))] for x0 in range(h)]
    sg = -1.0 if d % 2 else 1.0
    high = [[sg * w for w in lw[::-1]] for lw in low]
    return Operator(L, -h, inner, low, high, bl, bl, 0)


def centered_nonuniform(d: int, p: int, x: Sequence[float]) -> Operator:
    """``CompleteCenteredDifference(d, p, x::AbstractVector)``
    (centered_difference/centered_diff_weights.jl:77-153): Fornberg weights on the grid's own
    nodes, one interior row per interior point; boundary rows on the first / last bL nodes
    taken relative to the first (resp. the one before the last bL) node, as the reference's
    cumulative sums of the spacings give them."""
    x = [float(v) for v in x]
    L = d + p - 1 + (d + p) % 2
    bl = d + p
    h = L // 2
    n = len(x)
    if n < bl + 1 or n < L:
        raise NotImplementedError("nonuniform grid too short for the stencil")
    dxv = [x[i + 1] - x[i] for i in range(n - 1)]
    rows = [fornberg(d, x[i], x[i - h:i + h + 1]) for i in range(h, n - h)]
    low_x = [0.0]
    for v in dxv[:bl - 1]:
        low_x.append(low_x[-1] + v)
    high_x = []
    acc = 0.0
    for k, v in enumerate(dxv[n - 1 - bl:]):
        acc = v if k == 0 else acc + v
        high_x.append(acc)
    low = [fornberg(d, low_x[i], low_x) for i in range(h)]
    high = [fornberg(d, high_x[bl - 1 - i], high_x) for i in range(h)]
    return Operator(L, -h, rows[0], low, high, bl, bl, 0, rows)


def upwind(d: int, p: int, dx: float, offside: int) -> Operator:
    L = d + p
    bl = d + p
    s = 1.0 / julia_pow(dx, d)
    inner = [s * w for w in fornberg(d, 0.0, [float(k - offside) for k in range(L)])]
    low = [[s * w for w in fornberg(d, float(x0), [float(k) for k in range(bl)])] for x0 in range(offside)]
    nhi = L - 1 - offside
    neg = -1.0 / dx
    hs = julia_pow(neg, d) if d <= 3 else float(Fraction(neg) ** d)
    hx = [-float(k) for k in range(bl)]
    high = [[hs * w for w in fornberg(d, -float(k), hx)] for k in range(nhi)][::-1]
    return Operator(L, -offside, inner, low, high, bl, bl, 0)


def upwind_nonuniform(d: int, p: int, x: Sequence[float], offside: int) -> Operator:
    """``CompleteUpwindDifference(d, p, x::AbstractVector, offside)``
    (upwind_difference/upwind_diff_weights.jl:93-171) in the form its tap selection reads it
    (upwind_difference.jl:131-162): the reference returns the operator with offside 0, so a
    point i uses the i-th table row (built for the point i + offside) with taps i .. i+L-1
    (offside 0) or i-L+1 .. i (offside L-1), and only the offside-0 operator has high rows
    (weights at the last L-1 points, in grid order, on the last bL nodes, the first of them
    used at the last point).  Rows as in the reference; only L = 2 reaches no further than
    its table on every interior point."""
    x = [float(v) for v in x]
    L = d + p
    bl = d + p
    nlo = offside
    nhi = L - 1 - offside
    n = len(x)
    rows = [fornberg(d, x[i - 1], x[i - 1 - offside:i - 1 + L - offside]) for i in range(nlo + 1, n - nhi + 1)]
    high = [fornberg(d, x0, x[n - bl:]) for x0 in x[n - nhi:]] if (offside == 0 and nhi > 0) else []
    omin = 0 if offside == 0 else -(L - 1)
    return Operator(L, omin, rows[0], [], high, bl, bl, 0, rows)


def half_centered(d: int, p: int, dx: float) -> Operator:
    L = p + 2 * (d // 2) + (p % 2)
    bl = d + p
    e = L // 2
    s = 1.0 / julia_pow(dx, d)
    inner = [s * w for w in fornberg(d, 0.5, range(1 - e, e + 1))]
    low = [[s * w for w in fornberg(d, 1.5 + k, range(1, bl + 1))] for k in range(e)]
    sg = -1.0 if d % 2 else 1.0
    high = [[sg * w for w in lw[::-1]] for lw in low]
    return Operator(L, 1 - e, inner, low, high, bl, bl, 1)


def half_centered_nonuniform(d: int, p: int, x: Sequence[float]) -> Operator:
    """``CompleteHalfCenteredDifference(d, p, x::AbstractVector)`` (half_offset_weights.jl:72-150):
    per-half-point rows on the grid's own nodes.  Half point i (1-based, between nodes i and
    i+1) sits at (x_i + x_{i+1})/2; its interior row is Fornberg on nodes i-e+1 .. i+e (e half
    the stencil length), the low rows (half points 1..e) and high rows (the last e, last first)
    on the first / last d+p nodes.  Tap selection reads row i-e for half point i
    (half_offset_centred_difference.jl:39-69), the device's row index i - nlo - 1."""
    if p <= 1:
        raise ValueError("approximation_order must be greater than 1.")
    x = [float(v) for v in x]
    L = p + 2 * (d // 2) + (p % 2)
    bl = d + p
    e = L // 2
    n = len(x)
    if n < bl or n < L:
        raise NotImplementedError("nonuniform grid too short for the half-offset stencil")
    mid = [(x[k] + x[k + 1]) / 2 for k in range(n - 1)]
    rows = [fornberg(d, mid[i - 1], x[i - e:i + e]) for i in range(e + 1, n - e + 1)]
    low = [fornberg(d, mid[k], x[:bl]) for k in range(e)]
    high = [fornberg(d, mid[n - 2 - k], x[n - bl:]) for k in range(e)]
    if not rows:
        raise NotImplementedError("nonuniform grid too short for the half-offset stencil")
    return Operator(L, 1 - e, rows[0], low, high, bl, bl, 1, rows)


def extrapolator(q: int) -> Operator:
    """``BoundaryInterpolatorExtrapolator(q, dx)`` (extrapolation_weights.jl:1-60): row k of the
    low table gives the value at node k (0-based) of the first q nodes from the other q - 1
    (order-0 Fornberg weights, a zero in its own slot); the high rows are the low rows
    reversed.  No dx scaling: interpolation weights do not depend on the spacing."""
    L = q - 1 + q % 2
    h = L // 2
    low = []
    for x0 in range(h):
        others = [float(v) for v in range(q) if v != x0]
        w = fornberg(0, float(x0), others)
        low.append(w[:x0] + [0.0] + w[x0:])
    mid = [float(v) for v in range(-h, h + 1) if v != 0]
    wi = fornberg(0, 0.0, mid)
    interior = wi[:h] + [0.0] + wi[h:]
    return Operator(L, -h, interior, low, [lw[::-1] for lw in low], q, q, 0)


# ---------------------------------------------------------------------------------------
# Node-centred Lagrange WENO-5 on nonuniform grids (WENO/nonuniform_weno.jl:1-212): the
# geometry of every point (Fornberg three-point weights of the Simpson cell, the cell width,
# the split ideal weights) depends on the grid only and is tabulated here, in the
# reference's operation order; the device forms the smoothness indicators and nonlinear
# weights from the state.

WENO_NU_ROW = 56   # dx/6, dx, dx^3, then per substencil m1(xi), m1(xL), m1(xM), m1(xph), m2(xM),
                   # then dp_k/sigma_p, dm_k/sigma_m (k = 0..2), sigma_p, sigma_m


def _fb3(a, xt):
    """Three-point Fornberg weights (m = 1 and m = 2) at xt, _fornberg3_weights's order."""
    a0, a1, a2 = a
    c2 = a1 - a0
    r1 = 1.0 / c2
    tA = a1 - xt
    p1 = [(tA * 1.0) / c2, (tA * 0.0 - 1.0) / c2, (tA * 0.0 - 2 * 0.0) / c2]
    sB = a0 - xt
    p2 = [r1 * (-(sB) * 1.0), r1 * (1.0 - sB * 0.0), r1 * (2 * 0.0 - sB * 0.0)]
    c1 = c2
    c2 = (a2 - a0) * (a2 - a1)
    r2 = c1 / c2
    c3a, c3b = a2 - a0, a2 - a1
    tA2 = a2 - xt
    b1 = [(tA2 * p1[0]) / c3a, (tA2 * p1[1] - p1[0]) / c3a, (tA2 * p1[2] - 2 * p1[1]) / c3a]
    b2 = [(tA2 * p2[0]) / c3b, (tA2 * p2[1] - p2[0]) / c3b, (tA2 * p2[2] - 2 * p2[1]) / c3b]
    sB2 = a1 - xt
    b3 = [r2 * (-(sB2) * p2[0]), r2 * (p2[0] - sB2 * p2[1]), r2 * (2 * p2[1] - sB2 * p2[2])]
    return [b1[1], b2[1], b3[1]], [b1[2], b2[2], b3[2]]


def weno_nonuniform_target(i: int, n: int) -> Tuple[int, int]:
    """(first tap, target) at 1-based point i of n: two one-sided targets at each end, the
    centre elsewhere (get_f_taps_coords, function_scheme.jl:1-34; WENO.jl:84-85)."""
    if i <= 2:
        return 1, i
    if i > n - 2:
        return n - 4, 5 - (n - i)
    return i - 2, 3


def weno_nonuniform_rows(x: Sequence[float]) -> List[List[float]]:
    """One WENO_NU_ROW-vector per grid point (1-based point i in row i-1)."""
    x = [float(v) for v in x]
    n = len(x)
    rows = []
    for i in range(1, n + 1):
        q0, tg = weno_nonuniform_target(i, n)
        x1, x2, x3, x4, x5 = x[q0 - 1:q0 + 4]
        xi, xL, xph = {1: (x1, x1, (x1 + x2) / 2), 2: (x2, (x1 + x2) / 2, (x2 + x3) / 2),
                       3: (x3, (x2 + x3) / 2, (x3 + x4) / 2), 4: (x4, (x3 + x4) / 2, (x4 + x5) / 2),
                       5: (x5, (x4 + x5) / 2, x5)}[tg]
        dx = xph - xL
        xM = (xL + xph) / 2
        row = [dx / 6, dx, dx * dx * dx]
        for al in ((x1, x2, x3), (x2, x3, x4), (x3, x4, x5)):
            m1i, _ = _fb3(al, xi)
            m1L, _ = _fb3(al, xL)
            m1M, m2M = _fb3(al, xM)
            m1R, _ = _fb3(al, xph)
            row += m1i + m1L + m1M + m1R + m2M
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
        d1 = 1.0 - d0 - d2
        dp = [0.5 * (d + 3.0 * abs(d)) for d in (d0, d1, d2)]
        dm = [dp[0] - d0, dp[1] - d1, dp[2] - d2]
        sp_ = dp[0] + dp[1] + dp[2]
        sm_ = dm[0] + dm[1] + dm[2]
        row += [v / sp_ for v in dp] + [v / sm_ for v in dm] + [sp_, sm_]
        rows.append(row)
    return rows


def select(op: Operator, i: int, length: int, periodic: bool) -> Tuple[List[float], List[int]]:
    """(weights, unwrapped taps) of `op` at 1-based position i on a line of `length` points."""
    if not periodic and i <= op.nlo:
        return op.low[i - 1], list(range(1, op.bLlo + 1))
    if not periodic and i > length - op.nhi:
        return op.high[length - i - op.hi_base], list(range(length - op.bLhi + 1, length + 1))
    w = op.rows[i - op.nlo - 1] if op.rows is not None else op.interior
    return w, list(range(i + op.omin, i + op.omin + op.L))


def wrap(i: int, l: int) -> int:
    """Periodic index wrap, u[1] == u[l] (interface_boundary.jl:33-42)."""
    if i <= 1:
        return i + (l - 1)
    if i > l:
        return i - (l - 1)
    return i
