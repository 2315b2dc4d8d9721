"""The oracle's WENO restatements against the reference's own WENO tests (no device needed).

The assertions are those of ``test/Components/weno_nonuniform_core.jl`` (node-centred
Lagrange WENO-5 on nonuniform grids) and ``test/Components/weno_dispatch.jl`` (the uniform
Jiang-Shu WENO5 on the inputs that test uses), applied to ``oracle/weno_nonuniform.py`` and
``oracle/mol_oracle.weno5`` with the reference's points, functions and tolerances.
"""
import math

import numpy as np
import pytest

from oracle.mol_oracle import weno5
from oracle.weno_nonuniform import fornberg3_weights, ideal_d0d2, weno_f_nonuniform

EPS = 1.0e-6


def wf(u, x):
    return weno_f_nonuniform(list(u), EPS, list(x), 3)


def ideal_weights(x):
    d0, d2 = ideal_d0d2(3, *x)
    return d0, 1.0 - d0 - d2, d2


def sub_deriv(al, ua, ub, uc, xt):
    _, w1, _ = fornberg3_weights(al, xt)
    return w1[0] * ua + w1[1] * ub + w1[2] * uc


def linear_recon(x, u):
    """sum_k d_k p_k'(x_3): the linear (ideal-weight) reconstruction, weno_nonuniform_core.jl:44-51."""
    d0, d1, d2 = ideal_weights(x)
    r0 = sub_deriv((x[0], x[1], x[2]), u[0], u[1], u[2], x[2])
    r1 = sub_deriv((x[1], x[2], x[3]), u[1], u[2], u[3], x[2])
    r2 = sub_deriv((x[2], x[3], x[4]), u[2], u[3], u[4], x[2])
    return d0 * r0 + d1 * r1 + d2 * r2


def test_polynomial_exactness_degree_2():
    """weno_nonuniform_core.jl:55-73."""
    xs = [0.0, 0.6, 1.4, 2.1, 3.3]
    xc = xs[2]
    f0, df0 = (lambda x: 1.7), 0.0
    f1, df1 = (lambda x: 1.7 + 0.9 * x), 0.9
    f2, df2 = (lambda x: 1.7 + 0.9 * x - 0.4 * x ** 2), 0.9 - 0.8 * xc
    assert abs(wf([f0(x) for x in xs], xs) - df0) <= 1e-14
    assert abs(wf([f1(x) for x in xs], xs) - df1) <= 1e-13
    assert abs(wf([f2(x) for x in xs], xs) - df2) <= 1e-12
    # not exact for degree 3 at finite h
    assert abs(wf([x ** 3 for x in xs], xs) - 3 * xc ** 2) > 1e-6


@pytest.mark.parametrize("xs", [[0.0, 0.6, 1.4, 2.1, 3.3], [-0.3, 0.4, 0.55, 1.9, 2.4]])
def test_linear_ideal_weight_identity_degree_4(xs):
    """weno_nonuniform_core.jl:75-91: the ideal weights are a convex partition and their
    linear reconstruction is exact through degree 4."""
    xc = xs[2]
    d0, d1, d2 = ideal_weights(xs)
    assert abs(d0 + d1 + d2 - 1.0) <= 1e-14
    assert all(0 <= d <= 1 for d in (d0, d1, d2))
    for g, dg in ((lambda x: x ** 3 - 2 * x, lambda x: 3 * x ** 2 - 2),
                  (lambda x: x ** 4 - 0.5 * x ** 2 + x, lambda x: 4 * x ** 3 - x + 1),
                  (lambda x: 2.3 * x ** 4 - 1.1 * x ** 3, lambda x: 9.2 * x ** 3 - 3.3 * x ** 2)):
        got, want = linear_recon(xs, [g(x) for x in xs]), dg(xc)
        assert abs(got - want) <= 1e-11 + 1e-11 * abs(want)


def test_order_of_convergence():
    """weno_nonuniform_core.jl:93-114: self-similar refinement of a fixed offset pattern."""
    f = lambda x: math.sin(1.3 * x) + 0.5 * x
    df = lambda x: 1.3 * math.cos(1.3 * x) + 0.5
    o = [-2.0, -1.13, 0.08, 0.91, 2.0]
    xc = 1.0
    hs = [0.2, 0.1, 0.05, 0.025, 0.0125]
    errs = []
    for h in hs:
        xs = [xc + h * v for v in o]
        errs.append(abs(wf([f(x) for x in xs], xs) - df(xs[2])))
    orders = [math.log2(errs[k] / errs[k + 1]) for k in range(len(hs) - 1)]
    assert orders[-1] > 3.85
    assert orders[-2] > 3.7
    lh = np.log(hs[2:])
    le = np.log(errs[2:])
    n = len(lh)
    slope = (n * np.sum(lh * le) - np.sum(lh) * np.sum(le)) / (n * np.sum(lh ** 2) - np.sum(lh) ** 2)
    assert slope > 3.8
    assert all(v > 3.0 for v in orders)


@pytest.mark.parametrize("g", [[0.0, 1.0, 1.0 + 1.0e-6, 2.0 + 1.0e-6, 3.0 + 1.0e-6],
                               [0.0, 1.0e-6, 2.0e-6, 1.0, 2.0]])
def test_extreme_grid_stretching(g):
    """weno_nonuniform_core.jl:116-144: finite, exact for a linear field, bounded for a
    quadratic, finite convex-sum ideal weights with d1 >= 0."""
    assert math.isfinite(wf([x ** 2 for x in g], g))
    lin = wf([2.0 + 3.0 * x for x in g], g)
    assert abs(lin - 3.0) <= 1e-6 * 3.0
    assert abs(wf([x ** 2 for x in g], g) - 2 * g[2]) < 1.0
    d0, d1, d2 = ideal_weights(g)
    assert all(math.isfinite(d) for d in (d0, d1, d2))
    assert d1 >= 0
    assert abs(d0 + d1 + d2 - 1.0) <= 1e-10


def test_stretching_sweep_stays_finite():
    """weno_nonuniform_core.jl:136-143: spacing ratios 1e-3 .. 1e3."""
    for k in range(61):
        s = 10.0 ** (k / 10 - 3)
        g = list(np.cumsum([1.0, s, 1.0, s, 1.0]) - 1.0)
        assert math.isfinite(wf([math.sin(x) for x in g], g)), k


def test_derivative_in_u3_matches_central_difference():
    """weno_nonuniform_core.jl:167-200 checks d/du_3 (forward-mode AD) against a central
    difference with h = 1e-6 at rtol 1e-5.  Without AD here: central differences at h and h/2
    agree to that tolerance (the function is smooth in u_3 at this point)."""
    xs = [0.0, 0.6, 1.4, 2.1, 3.3]
    u = [1.7 + 0.9 * x - 0.4 * x ** 2 for x in xs]

    def dfd(h):
        up, um = list(u), list(u)
        up[2] += h
        um[2] -= h
        return (wf(up, xs) - wf(um, xs)) / (2 * h)

    assert abs(dfd(1e-6) - dfd(5e-7)) <= 1e-5 * abs(dfd(1e-6))


def test_uniform_weno5_on_the_dispatch_inputs():
    """weno_dispatch.jl:7-16 evaluates the uniform WENO at u = 1..5, eps = 1e-6, dx = 0.1 (and
    checks that the generic entry point agrees with it): for linear data every candidate
    reconstruction is exact, so the value is the slope 10 up to rounding, and the nonuniform
    core on the same uniform nodes agrees."""
    u = [1.0, 2.0, 3.0, 4.0, 5.0]
    v = weno5(*u, EPS, 0.1)
    assert abs(v - 10.0) <= 1e-12
    x = [0.0, 0.1, 0.2, 0.30000000000000004, 0.4]
    assert abs(wf(u, x) - 10.0) <= 1e-12
