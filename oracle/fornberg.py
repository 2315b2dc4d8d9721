"""Oracle restatement of MethodOfLines.jl's finite-difference weight tables.

Every function reproduces the reference's Float64 operation order so that the
weights come out bit-identical (Python floats are IEEE binary64 and Python does
not contract multiply-adds, exactly like Julia without ``@fastmath``).

Test infrastructure only: imported by tests and the CPU baseline, never by the
product package.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from fractions import Fraction
from typing import List, Sequence


def calculate_weights(order: int, x0: float, x: Sequence[float]) -> List[float]:
    """Fornberg (1988) weights, ``src/discretization/schemes/fornberg_calculate_weights.jl:20-65``.

    Integer node coordinates are converted exactly (Julia promotes ``Int`` to
    ``Float64`` inside the same expressions).  The sum-to-zero correction of the
    middle weight (``:62-65``) is applied for ``order != 0``; the sum is a
    left-to-right fold, which is what Julia's ``sum`` does below 16 elements.
    """
    N = len(x)
    assert order < N, "Not enough points for the requested order."
    M = order
    x = [float(v) for v in x]
    x0 = float(x0)
    c1 = 1.0
    c4 = x[0] - x0
    C = [[0.0] * (M + 1) for _ in range(N)]
    C[0][0] = 1.0
    for i in range(1, N):            # Julia i in 1:N-1, i1 = i+1 -> python row i
        mn = min(i, M)
        c2 = 1.0
        c5 = c4
        c4 = x[i] - x0
        for j in range(0, i):        # Julia j in 0:i-1, j1 = j+1 -> python row j
            c3 = x[i] - x[j]
            c2 *= c3
            if j == i - 1:
                for s in range(mn, 0, -1):
                    C[i][s] = c1 * (s * C[i - 1][s - 1] - c5 * C[i - 1][s]) / c2
                C[i][0] = -c1 * c5 * C[i - 1][0] / c2
            for s in range(mn, 0, -1):
                C[j][s] = (c4 * C[j][s] - s * C[j][s - 1]) / c3
            C[j][0] = c4 * C[j][0] / c3
        c1 = c2
    out = [C[k][M] for k in range(N)]
    if order != 0:
        if N < 16:
            acc = out[0] + out[1] if N >= 2 else out[0]
            for k in range(2, N):
                acc = acc + out[k]
        else:  # pragma: no cover - stencils here are short
            acc = _pairwise_sum(out)
        out[N // 2] -= acc
    return out


def _pairwise_sum(v):
    if len(v) <= 16:
        acc = v[0]
        for a in v[1:]:
            acc = acc + a
        return acc
    h = len(v) // 2
    return _pairwise_sum(v[:h]) + _pairwise_sum(v[h:])


def dx_pow(dx: float, d: int) -> float:
    """``dx^d`` as Julia's ``^(::Float64, ::Int)`` gives it for d <= 3.

    d = 2 is the correctly rounded square (Julia's compensated power returns
    fl(dx*dx)), d = 3 is ``dx*dx*dx`` (Julia's explicit n == 3 branch).  For
    d >= 4 the correctly rounded power is returned; Julia's compensated
    power-by-squaring agrees in the overwhelming majority of cases but this is
    not pinned.
    """
    if d == 0:
        return 1.0
    if d == 1:
        return dx
    if d == 2:
        return dx * dx
    if d == 3:
        return dx * dx * dx
    return float(Fraction(dx) ** d)


@dataclass
class DerivativeOperator:
    """Field subset of ``src/discretization/derivative_operator.jl:1-15``."""
    derivative_order: int
    approximation_order: int
    dx: float
    stencil_length: int
    stencil_coefs: List[float]
    boundary_stencil_length: int
    boundary_point_count: int
    low_boundary_coefs: List[List[float]]
    high_boundary_coefs: List[List[float]]
    offside: int = 0
    kind: str = "centered"


def _scale(s: float, w):
    return [s * v for v in w]


def complete_centered_difference(d: int, p: int, dx: float) -> DerivativeOperator:
    """``CompleteCenteredDifference``, ``centered_difference/centered_diff_weights.jl:4-75``."""
    assert p > 1
    L = d + p - 1 + (d + p) % 2
    bL = d + p
    half = L // 2
    dummy_x = list(range(-half, half + 1))
    left_x = list(range(0, bL))
    bpc = half
    spots = left_x[:half]
    s = 1.0 / dx_pow(dx, d)
    stencil = _scale(s, calculate_weights(d, 0.0, dummy_x))
    low = [_scale(s, calculate_weights(d, 1.0 * x0, left_x)) for x0 in spots]
    sign = -1.0 if d % 2 else 1.0
    high = [[v * sign for v in reversed(w)] for w in low]
    return DerivativeOperator(d, p, dx, L, stencil, bL, bpc, low, high, 0, "centered")


def complete_centered_difference_nonuniform(d: int, p: int, x: Sequence[float]) -> DerivativeOperator:
    """``CompleteCenteredDifference(d, p, x::AbstractVector)``,
    ``centered_difference/centered_diff_weights.jl:77-153``.

    ``stencil_coefs`` is then a list with one row per interior point (points
    bpc+1 .. len-bpc, 1-based), each the Fornberg weights at x[i] on x[i-bpc .. i+bpc].
    The boundary rows use node coordinates rebuilt from the spacings: the low rows
    ``[0; cumsum(dx[1:bL-1])]`` evaluated at their first bpc nodes, the high rows
    ``cumsum(dx[end-bL+1:end])`` evaluated at their last bpc nodes, last node first.
    ``cumsum`` of a Vector is a sequential left fold.  No 1/dx^d scaling: the nodes carry
    the physical coordinates.
    """
    x = [float(v) for v in x]
    L = d + p - 1 + (d + p) % 2
    bL = d + p
    bpc = L // 2
    n = len(x)
    dxs = [x[i + 1] - x[i] for i in range(n - 1)]

    def cumsum(v):
        out, acc = [], None
        for a in v:
            acc = a if acc is None else acc + a
            out.append(acc)
        return out

    low_x = [0.0] + cumsum(dxs[:bL - 1])
    high_x = cumsum(dxs[len(dxs) - bL:])
    stencil = [calculate_weights(d, x[i - 1], x[i - 1 - bpc:i + bpc]) for i in range(bpc + 1, n - bpc + 1)]
    low = [calculate_weights(d, low_x[k], low_x) for k in range(bpc)]
    high = [calculate_weights(d, high_x[len(high_x) - 1 - k], high_x) for k in range(bpc)]
    return DerivativeOperator(d, p, float("nan"), L, stencil, bL, bpc, low, high, 0, "centered_nonuniform")


def boundary_interpolator_extrapolator(q: int, dx: float) -> DerivativeOperator:
    """``BoundaryInterpolatorExtrapolator(q, dx)``, ``extrapolation_weights.jl:1-60``.

    ``remove`` drops the node itself from the node list and ``insert`` puts a zero weight
    back in its slot; the high rows are the low rows reversed.
    """
    L = q - 1 + q % 2
    bL = q
    half = L // 2
    dummy_x = list(range(-half, half + 1))
    left_x = list(range(0, bL))
    bpc = half

    def remove(v, x):
        return [a for a in v if a != x]

    def insert(v, i, val):          # Julia's insert!(v, i, val), 1-based i
        return list(v[:i - 1]) + [val] + list(v[i - 1:])

    stencil = insert(calculate_weights(0, 0.0, remove(dummy_x, 0)), dummy_x.index(0) + 1, 0.0)
    low = [insert(calculate_weights(0, 1.0 * x0, remove(left_x, x0)), i, 0.0)
           for i, x0 in enumerate(left_x[:bpc], start=1)]
    high = [list(reversed(v)) for v in low]
    return DerivativeOperator(0, q, dx, L, stencil, bL, bpc, low, high, 0, "extrapolation")


def complete_upwind_difference(d: int, p: int, dx: float, offside: int = 0) -> DerivativeOperator:
    """``CompleteUpwindDifference``, ``upwind_difference/upwind_diff_weights.jl:4-91``."""
    assert offside > -1
    L = d + p
    bL = d + p
    nlo = offside
    nhi = L - 1 - offside
    dummy_x = [float(k) for k in range(-offside, L - offside)]
    s = 1.0 / dx_pow(dx, d)
    stencil = _scale(s, calculate_weights(d, 0.0, dummy_x))
    low_x = [float(k) for k in range(0, bL)]
    low = [_scale(s, calculate_weights(d, float(x0), low_x)) for x0 in range(0, nlo)]
    high_x = [-float(k) for k in range(0, bL)]
    neg = -1.0 / dx
    hs = 1.0
    if d == 1:
        hs = neg
    elif d == 2:
        hs = neg * neg
    elif d == 3:
        hs = neg * neg * neg
    elif d > 3:
        hs = float(Fraction(neg) ** d)
    _high = [_scale(hs, calculate_weights(d, -float(k), high_x)) for k in range(0, nhi)]
    high = list(reversed(_high))
    # upwind operators report the high point count as boundary_point_count
    return DerivativeOperator(d, p, dx, L, stencil, bL, nhi, low, high, offside, "upwind")


def complete_upwind_difference_nonuniform(d: int, p: int, x: Sequence[float], offside: int = 0) -> DerivativeOperator:
    """``CompleteUpwindDifference(d, p, x::AbstractVector, offside)``,
    ``upwind_difference/upwind_diff_weights.jl:93-171``.

    ``stencil_coefs[k]`` (0-based) holds the weights at x[i] on x[i - offside .. i + L - 1 -
    offside] for the grid point i = offside + 1 + k (1-based); the high rows are the weights
    at the last L - 1 - offside points, in grid order, on the last bL nodes.  As the
    reference returns it, the operator's ``offside`` is 0 and its boundary point count the
    high count: its tap selection (``_upwind_difference`` for DX <: AbstractVector,
    upwind_difference.jl:131-162) then reads ``stencil_coefs[II]`` for a point II, i.e. the
    row built for point II + offside.
    """
    x = [float(v) for v in x]
    L = d + p
    bL = d + p
    nlo = offside
    nhi = L - 1 - offside
    n = len(x)
    stencil = [calculate_weights(d, x[i - 1], x[i - 1 - offside:i - 1 + L - offside]) for i in range(nlo + 1, n - nhi + 1)]
    low_x = x[:bL]
    high_x = x[n - bL:]
    low = [calculate_weights(d, x0, low_x) for x0 in x[:nlo]]
    high = [calculate_weights(d, x0, high_x) for x0 in x[n - nhi:]] if nhi > 0 else []
    return DerivativeOperator(d, p, float("nan"), L, stencil, bL, nhi, low, high, 0, "upwind_nonuniform")


def complete_half_centered_difference_nonuniform(d: int, p: int, x: Sequence[float]) -> DerivativeOperator:
    """``CompleteHalfCenteredDifference(d, p, x::AbstractVector)``, ``half_offset_weights.jl:72-150``.

    With hx[i] = (x[i] + x[i+1]) / 2 the half points (1-based), ``stencil_coefs`` holds one
    row per half point i = endpoint+1 .. len(x)-endpoint: the Fornberg weights at hx[i] on
    x[i-endpoint+1 .. i+endpoint].  The low rows are the weights at hx[1..bpc] on the first
    bL nodes, the high rows the weights at hx[end], hx[end-1], ... on the last bL nodes.  No
    1/dx^d scaling: the nodes carry the physical coordinates.
    """
    assert p > 1
    x = [float(v) for v in x]
    L = p + 2 * (d // 2) + (p % 2)
    bL = d + p
    endpoint = L // 2
    n = len(x)
    hx = [(x[i] + x[i + 1]) / 2 for i in range(n - 1)]
    stencil = [calculate_weights(d, hx[i - 1], x[i - endpoint:i + endpoint]) for i in range(endpoint + 1, n - endpoint + 1)]
    low_x = x[:bL]
    high_x = x[n - bL:]
    low = [calculate_weights(d, off, low_x) for off in hx[:endpoint]]
    high = [calculate_weights(d, hx[len(hx) - 1 - k], high_x) for k in range(endpoint)]
    return DerivativeOperator(d, p, float("nan"), L, stencil, bL, endpoint, low, high, 0, "half_nonuniform")


def complete_half_centered_difference(d: int, p: int, dx: float) -> DerivativeOperator:
    """``CompleteHalfCenteredDifference``, ``half_offset_weights.jl:4-70``."""
    assert p > 1
    L = p + 2 * (d // 2) + (p % 2)
    bL = d + p
    endpoint = L // 2
    dummy_x = list(range(1 - endpoint, endpoint + 1))
    left_x = list(range(1, bL + 1))
    bpc = L // 2
    xoffset = [1.5 + k for k in range(bpc)]
    spots = xoffset[:L // 2]
    s = 1.0 / dx_pow(dx, d)
    stencil = _scale(s, calculate_weights(d, 0.5, dummy_x))
    low = [_scale(s, calculate_weights(d, off, left_x)) for off in spots]
    sign = -1.0 if d % 2 else 1.0
    high = [[v * sign for v in reversed(w)] for w in low]
    return DerivativeOperator(d, p, dx, L, stencil, bL, bpc, low, high, 0, "half")
