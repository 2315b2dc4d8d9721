"""Boundary rows on the GPU against the oracle: constant and time/parameter-dependent Robin
rows, Neumann, Dirichlet with data, in 1-D and 2-D, through the RHS, fixed SSPRK33 steps
and the discrete adjoint (reference: generate_bc_eqs.jl:238-328; the reference's
test/Diffusion/MOL_1D_Linear_Diffusion.jl exercises the same rows)."""
import math

import numpy as np
import pytest

from molgpu import Plan, lower
from molgpu.api import MOLFiniteDifference
from molgpu.symbolic import Differential, Eq, Field, Interval, IV, Param, PDESystem, cos, sin
from oracle.integrators import ssprk33
from oracle.mol_oracle import OracleProblem

pytestmark = pytest.mark.gpu


def _robin_1d(dynamic):
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    k = Param("k", 2.0)
    lo = k * t if dynamic else 1.0
    hi = t * t + 1.0 if dynamic else 0.5
    s = PDESystem([Eq(Dt(u(x, t)), Dxx(u(x, t)) - k * u(x, t) * u(x, t))],
                  [Eq(u(x, 0.0), 1.0 + 0.5 * sin(3.0 * x)), Eq(2.0 * u(0.0, t) + 3.0 * Dx(u(0.0, t)), lo),
                   Eq(Dx(u(1.0, t)), hi)],
                  [(t, Interval(0, 1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [k])
    return s.to_spec(MOLFiniteDifference({x: 0.05}, t))


def _mixed_2d():
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx, Dyy = Differential(t), Differential(x), Differential(x) ** 2, Differential(y) ** 2
    s = PDESystem([Eq(Dt(u(x, y, t)), Dxx(u(x, y, t)) + Dyy(u(x, y, t)) + 0.1 * u(x, y, t))],
                  [Eq(u(x, y, 0.0), 1.0 + 0.3 * cos(2.0 * x) * sin(3.0 * y)),
                   Eq(u(0.0, y, t) + 0.5 * Dx(u(0.0, y, t)), 1.0), Eq(Dx(u(1.0, y, t)), 0.0),
                   Eq(u(x, 0.0, t), 1.0), Eq(u(x, 1.0, t), 1.0 + t)],
                  [(t, Interval(0, 1)), (x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0))], [t, x, y],
                  [u(x, y, t)], [])
    return s.to_spec(MOLFiniteDifference({x: 1.0 / 24, y: 1.0 / 20}, t))


SPECS = {"robin_const_1d": lambda: _robin_1d(False), "robin_dynamic_1d": lambda: _robin_1d(True),
         "robin_neumann_dirichlet_2d": _mixed_2d}


@pytest.mark.parametrize("name", sorted(SPECS))
def test_boundary_rows_rhs_and_trajectory(gpu_lib, name):
    spec = SPECS[name]()
    lw = lower(spec)
    orc = OracleProblem(spec)
    plan = Plan(lw)
    v = lw.u0 + 0.05 * np.random.default_rng(4).standard_normal(lw.n_unknowns)
    for t in (0.0, 0.37):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, v, None, t)
        ref = orc.rhs(v, t)
        assert np.linalg.norm(du - ref) <= 1e-12 * np.linalg.norm(ref), (name, t)
    dx = min(lw.dx)
    dt = 0.2 * dx * dx
    u = lw.u0.copy()
    plan.step_ssprk33(u, dt, 30, t0=0.1)
    ref, _ = ssprk33(lambda w, tt: orc.rhs(w, tt), lw.u0, 0.1, dt, 30)
    assert np.linalg.norm(u - ref) <= 1e-10 * np.linalg.norm(ref), name
    plan.close()


@pytest.mark.parametrize("name", ["robin_const_1d", "robin_dynamic_1d"])
def test_boundary_rows_adjoint_matches_finite_differences(gpu_lib, name):
    """The transposed boundary rows (constant rows through the precomputed reciprocal, rows
    with programs through the generic path) in the discrete adjoint."""
    spec = SPECS[name]()
    lw = lower(spec)
    plan = Plan(lw)
    dt, n = 0.2 * min(lw.dx) ** 2, 25
    target = np.zeros(lw.n_unknowns)

    def loss(u0):
        u = u0.copy()
        plan.step_ssprk33(u, dt, n, t0=0.0)
        return 0.5 * float(np.sum((u - target) ** 2))

    g = np.zeros(lw.n_unknowns)
    plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=4, dLdu0=g)
    w = np.random.default_rng(9).standard_normal(lw.n_unknowns)
    h = 1e-6
    fd = (loss(lw.u0 + h * w) - loss(lw.u0 - h * w)) / (2 * h)
    assert abs(g @ w - fd) <= 1e-6 * abs(fd), (g @ w, fd)
    plan.close()


def test_registered_function_in_a_boundary_row_gpu(gpu_lib):
    """A registered function of coordinates in a Dirichlet row (the boundary-condition docs'
    example), host-evaluated on the boundary face and read by the row's program."""
    from test_lowering import _registered_bc_problem
    spec = _registered_bc_problem()
    lw = lower(spec)
    orc = OracleProblem(spec)
    plan = Plan(lw)
    v = lw.u0 + 0.05 * np.random.default_rng(4).standard_normal(lw.n_unknowns)
    for t in (0.0, 0.37):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, v, None, t)
        ref = orc.rhs(v, t)
        assert np.linalg.norm(du - ref) <= 1e-12 * np.linalg.norm(ref), t
    full = plan.fill_grid(v, 0.37)[0]
    assert np.allclose(full, orc.solution_arrays(v, 0.37, lw.param_values)["u"], rtol=1e-12, atol=1e-13)
    plan.close()
