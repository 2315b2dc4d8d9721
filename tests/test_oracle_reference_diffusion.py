"""The oracle's boundary rows against the reference's 1-D diffusion tests (no device needed).

``test/Diffusion/MOL_1D_Linear_Diffusion.jl`` solves u_t = u_xx with Neumann, mixed
Neumann/Dirichlet and Robin rows (constant and time-dependent coefficients), on center- and
edge-aligned grids, and compares sol[u(t, x)] (every grid point, the observed boundary values
included) with the manufactured solution at t = 0, 0.1, ..., 1.  The same systems are built
here with the front end, integrated through the oracle's right-hand side (SSPRK33 where the
reference uses Tsit5; scipy's Radau where it uses the implicit Rodas4) and checked at the
reference's tolerances on the oracle's solution arrays.
"""
import math

import numpy as np
import pytest

from molgpu.api import MOLFiniteDifference
from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, cos, exp, sin
from oracle.integrators import ssprk33
from oracle.mol_oracle import OracleProblem

SAVE = [0.1 * k for k in range(11)]


def _system(bcs_of, lo, hi):
    x, t = IV("x"), IV("t")
    u = Field("u")
    eq = Eq(Differential(t)(u(x, t)), (Differential(x) ** 2)(u(x, t)))
    return PDESystem([eq], bcs_of(x, t, u, Differential(x)), [(t, Interval(0.0, 1.0)), (x, Interval(lo, hi))],
                     [t, x], [u(x, t)], []), x, t


def _explicit(orc, dt_frac):
    """sol[u] at SAVE by SSPRK33 with dt = dt_frac dx^2 (a whole number of steps per save)."""
    u = orc.initial_condition()
    dx = orc.dx[0]
    out = [orc.solution_arrays(u, 0.0, orc.param_values)["u"]]
    t = 0.0
    for k in range(1, len(SAVE)):
        n = int(math.ceil((SAVE[k] - t) / (dt_frac * dx * dx)))
        u, _ = ssprk33(lambda v, s: orc.rhs(v, s), u, t, (SAVE[k] - t) / n, n)
        t = SAVE[k]
        out.append(orc.solution_arrays(u, t, orc.param_values)["u"])
    return out


def _implicit(orc, rtol):
    """sol[u] at SAVE by scipy's Radau (the reference integrates these with Rodas4); the
    finite-difference Jacobian is grouped by a band that covers the stencils and the observed
    boundary values' one-sided rows."""
    integ = pytest.importorskip("scipy.integrate")
    sparse = pytest.importorskip("scipy.sparse")
    n = orc.n_unknowns
    band = sparse.diags([np.ones(n - abs(k)) for k in range(-12, 13)], list(range(-12, 13)), shape=(n, n))
    r = integ.solve_ivp(lambda s, v: orc.rhs(v, s), (0.0, 1.0), orc.initial_condition(), method="Radau",
                        t_eval=SAVE, rtol=rtol, atol=rtol * 1e-2, jac_sparsity=band)
    assert r.success
    return [orc.solution_arrays(r.y[:, k], SAVE[k], orc.param_values)["u"] for k in range(len(SAVE))]


def _check(orc, sols, exact, atol):
    xs = orc.grid[0]
    for k, s in enumerate(sols):
        err = np.max(np.abs(s - exact(xs, SAVE[k])))
        assert err <= atol, (SAVE[k], err)


def _trapezoid(xs):
    w = np.zeros(len(xs))
    h = np.diff(xs)
    w[:-1] += h / 2
    w[1:] += h / 2
    return w


def _exact_flow(orc):
    """sol[u] at SAVE for a linear homogeneous system du/dt = A u, A assembled column by column
    from the oracle's right-hand side, by the matrix exponential (the reference integrates with
    Tsit5 at tolerances 1e-10)."""
    linalg = pytest.importorskip("scipy.linalg")
    n = orc.n_unknowns
    assert not np.any(orc.rhs(np.zeros(n), 0.0))
    A = np.stack([orc.rhs(e, 0.0) for e in np.eye(n)], axis=1)
    u0 = orc.initial_condition()
    return [orc.solution_arrays(linalg.expm(A * s) @ u0, s, orc.param_values)["u"] for s in SAVE]


@pytest.mark.parametrize("align", ["center", "edge"])
def test_03_homogeneous_neumann_conserves_mass(align):
    """MOL_1D_Linear_Diffusion.jl:179-251: u_x = 0 at 0 and pi, 300 points; atol 0.01 at every
    point, and the trapezoidal integral of sol[u] over the grid stays at its initial value to
    1e-9."""
    sys_, x, t = _system(lambda x, t, u, Dx: [Eq(u(x, 0.0), cos(x)), Eq(Dx(u(0.0, t)), 0.0),
                                               Eq(Dx(u(math.pi, t)), 0.0)], 0.0, math.pi)
    dx = math.pi / 299
    orc = OracleProblem(sys_.to_spec(MOLFiniteDifference({x: dx}, t, grid_align=align)))
    sols = _exact_flow(orc)
    _check(orc, sols, lambda xs, s: math.exp(-s) * np.cos(xs), 0.01)
    w = _trapezoid(orc.grid[0])
    m0 = float(w @ sols[0])
    for s in sols:
        assert abs(float(w @ s) - m0) <= 1e-9


@pytest.mark.parametrize("align", ["center", "edge"])
def test_03a_inhomogeneous_neumann(align):
    """MOL_1D_Linear_Diffusion.jl:253-322: u_x = e^-t at 0 and -e^-t at pi, 30 points,
    approx_order 2; atol 0.01 at every point, and the rectangle-rule mass tracks its exact
    change 2 (e^-t - 1) to 0.01."""
    sys_, x, t = _system(lambda x, t, u, Dx: [Eq(u(x, 0.0), sin(x)), Eq(Dx(u(0.0, t)), exp(-1.0 * t)),
                                               Eq(Dx(u(math.pi, t)), -1.0 * exp(-1.0 * t))], 0.0, math.pi)
    dx = (math.pi - 0.0) / 29
    orc = OracleProblem(sys_.to_spec(MOLFiniteDifference({x: dx}, t, approx_order=2, grid_align=align)))
    sols = _explicit(orc, 0.2)
    _check(orc, sols, lambda xs, s: math.exp(-s) * np.sin(xs), 0.01)
    mass0 = float(np.sum(sols[0]) * dx)
    for k, s in enumerate(sols):
        assert abs(mass0 + 2 * (math.exp(-SAVE[k]) - 1) - float(np.sum(s) * dx)) <= 0.01


def test_04_neumann_and_dirichlet():
    """MOL_1D_Linear_Diffusion.jl:324-372: u = 0 at 0, u_x = -e^-t at pi, 30 points; atol 0.01."""
    sys_, x, t = _system(lambda x, t, u, Dx: [Eq(u(x, 0.0), sin(x)), Eq(u(0.0, t), 0.0),
                                               Eq(Dx(u(math.pi, t)), -1.0 * exp(-1.0 * t))], 0.0, math.pi)
    orc = OracleProblem(sys_.to_spec(MOLFiniteDifference({x: math.pi / 29}, t)))
    _check(orc, _explicit(orc, 0.2), lambda xs, s: math.exp(-s) * np.sin(xs), 0.01)


@pytest.mark.parametrize("align", ["center", "edge"])
def test_05_robin_order_4(align):
    """MOL_1D_Linear_Diffusion.jl:374-427: u + 3 u_x at -1 and 4 u + u_x at 1 with the exact
    solution's data, dx = 0.01, approx_order 4, implicit integration; atol 0.1."""
    def bcs(x, t, u, Dx):
        return [Eq(u(x, 0.0), sin(x)),
                Eq(u(-1.0, t) + 3.0 * Dx(u(-1.0, t)), exp(-1.0 * t) * (math.sin(-1.0) + 3.0 * math.cos(-1.0))),
                Eq(4.0 * u(1.0, t) + Dx(u(1.0, t)), exp(-1.0 * t) * (4.0 * math.sin(1.0) + math.cos(1.0)))]
    sys_, x, t = _system(bcs, -1.0, 1.0)
    orc = OracleProblem(sys_.to_spec(MOLFiniteDifference({x: 0.01}, t, approx_order=4, grid_align=align)))
    _check(orc, _implicit(orc, 1e-6), lambda xs, s: math.exp(-s) * np.sin(xs), 0.1)


def test_06_time_dependent_robin_order_6():
    """MOL_1D_Linear_Diffusion.jl:429-477: t^2 u + 3 u_x at -1 and 4 u + t u_x at 1, dx = 0.01,
    approx_order 6, implicit integration at reltol 1e-6; atol 0.06."""
    def bcs(x, t, u, Dx):
        return [Eq(u(x, 0.0), sin(x)),
                Eq(t * t * u(-1.0, t) + 3.0 * Dx(u(-1.0, t)),
                   exp(-1.0 * t) * (t * t * math.sin(-1.0) + 3.0 * math.cos(-1.0))),
                Eq(4.0 * u(1.0, t) + t * Dx(u(1.0, t)), exp(-1.0 * t) * (4.0 * math.sin(1.0) + t * math.cos(1.0)))]
    sys_, x, t = _system(bcs, -1.0, 1.0)
    orc = OracleProblem(sys_.to_spec(MOLFiniteDifference({x: 0.01}, t, approx_order=6)))
    _check(orc, _implicit(orc, 1e-6), lambda xs, s: math.exp(-s) * np.sin(xs), 0.06)


def _nonlinear(coef, exact, order=2, dirichlet=True, deriv=None):
    """u_t = Dx(a(u) Dx(u)) on [0, 2], dx = 0.01, data from the exact solution (Dirichlet, or
    Neumann with its derivative), integrated implicitly to t = 2 (the reference uses
    Rosenbrock32); returns the oracle's sol[u] at t = 2 and the exact values on the grid."""
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dx = Differential(x)
    U = u(x, t)
    eq = Eq(Differential(t)(U), Dx(coef(U) * Dx(U)))
    if dirichlet:
        bcs = [Eq(u(x, 0.0), exact(0.0, x)), Eq(u(0.0, t), exact(t, 0.0)), Eq(u(2.0, t), exact(t, 2.0))]
    else:
        bcs = [Eq(u(x, 0.0), exact(0.0, x)), Eq(Dx(u(0.0, t)), deriv(0.0)), Eq(Dx(u(2.0, t)), deriv(2.0))]
    sys_ = PDESystem([eq], bcs, [(t, Interval(0.0, 2.0)), (x, Interval(0.0, 2.0))], [t, x], [U], [])
    orc = OracleProblem(sys_.to_spec(MOLFiniteDifference({x: 0.01}, t, approx_order=order)))
    integ = pytest.importorskip("scipy.integrate")
    sparse = pytest.importorskip("scipy.sparse")
    n = orc.n_unknowns
    band = sparse.diags([np.ones(n - abs(k)) for k in range(-12, 13)], list(range(-12, 13)), shape=(n, n))
    r = integ.solve_ivp(lambda s, v: orc.rhs(v, s), (0.0, 2.0), orc.initial_condition(), method="Radau",
                        t_eval=[2.0], rtol=1e-6, atol=1e-8, jac_sparsity=band)
    assert r.success
    got = orc.solution_arrays(r.y[:, -1], 2.0, orc.param_values)["u"]
    xs = orc.grid[0]
    return got, np.array([exact(2.0, float(v)) for v in xs])


def test_nonlinear_00_inverse_coefficient():
    """Nonlinear_Diffusion/MOL_1D_NonLinear_Diffusion.jl:12-69: a(u) = u^-1, exact
    2 (1 + t) / (1 + x)^2, Dirichlet; the reference's isapprox on the arrays at t = 2 (2-norm of
    the difference within atol 0.1)."""
    got, want = _nonlinear(lambda U: U ** (-1), lambda t, x: 2.0 * (1.0 + t) / (1.0 + x) ** 2)
    assert np.linalg.norm(got - want) <= 0.1


@pytest.mark.parametrize("order", [2, 4])
def test_nonlinear_01_square_coefficient(order):
    """MOL_1D_NonLinear_Diffusion.jl:127-254 (Tests 01a and 01b): a(u) = u^2, exact
    0.5 (x + 0.5) / sqrt(50 - t), Dirichlet, approx_order 2 and 4; 2-norm within 0.1 at t = 2."""
    got, want = _nonlinear(lambda U: U ** 2, lambda t, x: 0.5 * (x + 0.5) / (50.0 - t) ** 0.5, order=order)
    assert np.linalg.norm(got - want) <= 0.1


def _two_d(rhs_of, order):
    """2-D/MOL_2D_Diffusion.jl: u on [0, 2]^2, dx = 0.1, dy = 0.2, Dirichlet data from
    exp(x + y) cos(x + y + 4t) on every side; sol[u] at t = 2 by an implicit solve through the
    oracle's right-hand side, and the exact values with the corners set to 0 as the test does."""
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    U = u(x, y, t)
    ex = lambda T, X, Y: exp(X + Y) * cos(X + Y + 4.0 * T)
    bcs = [Eq(u(x, y, 0.0), ex(0.0, x, y)), Eq(u(0.0, y, t), ex(t, 0.0, y)), Eq(u(2.0, y, t), ex(t, 2.0, y)),
           Eq(u(x, 0.0, t), ex(t, x, 0.0)), Eq(u(x, 2.0, t), ex(t, x, 2.0))]
    sys_ = PDESystem([Eq(Differential(t)(U), rhs_of(U, x, y, t))], bcs,
                     [(t, Interval(0.0, 2.0)), (x, Interval(0.0, 2.0)), (y, Interval(0.0, 2.0))], [t, x, y], [U], [])
    orc = OracleProblem(sys_.to_spec(MOLFiniteDifference({x: 0.1, y: 0.2}, t, approx_order=order)))
    integ = pytest.importorskip("scipy.integrate")
    r = integ.solve_ivp(lambda s, v: orc.rhs(v, s), (0.0, 2.0), orc.initial_condition(), method="Radau",
                        t_eval=[2.0], rtol=1e-6, atol=1e-8)
    assert r.success
    got = orc.solution_arrays(r.y[:, -1], 2.0, orc.param_values)["u"]
    X, Y = np.meshgrid(orc.grid[0], orc.grid[1], indexing="ij")
    want = np.exp(X + Y) * np.cos(X + Y + 8.0)
    want[0, 0] = want[0, -1] = want[-1, 0] = want[-1, -1] = 0.0
    assert got.shape == want.shape
    return got, want


def test_2d_00_heat_order_4():
    """MOL_2D_Diffusion.jl:8-73: u_t = u_xx + u_yy, approx_order 4; 2-norm of the difference
    at t = 2 within 0.4."""
    got, want = _two_d(lambda U, x, y, t: (Differential(x) ** 2)(U) + (Differential(y) ** 2)(U), 4)
    assert np.linalg.norm(got - want) <= 0.4


def test_2d_01_nonlinear_coefficient_of_coordinates_time_and_state():
    """MOL_2D_Diffusion.jl:75-149: a(x, y, t, u) = (u^2 / exp(x + y)^2 + sin(x + y + 4t)^2)^0.5
    (1 on the exact solution) in both nonlinear Laplacians; both sides scaled by the exact
    maximum, 2-norm within 0.4."""
    def rhs(U, x, y, t):
        a = (U ** 2 / exp(x + y) ** 2 + sin(x + y + 4.0 * t) ** 2) ** 0.5
        return Differential(x)(a * Differential(x)(U)) + Differential(y)(a * Differential(y)(U))
    got, want = _two_d(rhs, 2)
    m = np.max(want)
    assert np.linalg.norm(want / m - got / m) <= 0.4
