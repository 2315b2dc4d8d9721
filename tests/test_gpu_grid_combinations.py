"""Combinations of the grid and boundary variants (nonuniform WENO beside a periodic
dimension, a 3-D box with two nonuniform dimensions at order 4, an edge-aligned 2-D grid with
second-order upwinding and Robin rows, two coupled fields on a Chebyshev grid at order 6) on
the GPU: the generated RHS and fixed SSPRK33 steps against the oracle, and the discrete
adjoint against central differences for one of them."""
import numpy as np
import pytest

from molgpu import Plan, lower
from oracle.integrators import ssprk33
from oracle.mol_oracle import OracleProblem
from test_grid_combinations import CASES

pytestmark = pytest.mark.gpu


def _min_spacing(lw):
    return min(float(np.min(np.diff(g))) for g in lw.grids)


@pytest.mark.parametrize("name", sorted(CASES))
def test_combination_rhs_and_trajectory(gpu_lib, name):
    spec = CASES[name]()
    lw = lower(spec)
    orc = OracleProblem(spec)
    plan = Plan(lw)
    v = lw.u0 + 0.01 * np.random.default_rng(2).standard_normal(lw.n_unknowns)
    for t in (0.0, 0.41):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, v, None, t)
        ref = orc.rhs(v, t)
        assert np.linalg.norm(du - ref) <= 1e-12 * np.linalg.norm(ref), (name, t)
    dt, n = 0.1 * _min_spacing(lw) ** 2, 20
    u = lw.u0.copy()
    plan.step_ssprk33(u, dt, n, t0=0.05)
    ref, _ = ssprk33(lambda w, tt: orc.rhs(w, tt), lw.u0, 0.05, dt, n)
    assert np.linalg.norm(u - ref) <= 1e-10 * np.linalg.norm(ref), name
    plan.close()


def test_combination_adjoint_matches_finite_differences(gpu_lib):
    spec = CASES["edge_upwind_2d"]()
    lw = lower(spec)
    plan = Plan(lw)
    dt, n = 0.1 * _min_spacing(lw) ** 2, 16
    target = np.ones(lw.n_unknowns)

    def loss(u0):
        u = u0.copy()
        plan.step_ssprk33(u, dt, n, t0=0.0)
        return 0.5 * float(np.sum((u - target) ** 2))

    g = np.zeros(lw.n_unknowns)
    plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=4, dLdu0=g)
    w = np.random.default_rng(5).standard_normal(lw.n_unknowns)
    h = 1e-6
    fd = (loss(lw.u0 + h * w) - loss(lw.u0 - h * w)) / (2 * h)
    assert abs(g @ w - fd) <= 1e-6 * abs(fd), (g @ w, fd)
    plan.close()
