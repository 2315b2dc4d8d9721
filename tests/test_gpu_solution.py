"""Full-grid solution arrays on the GPU (mol_fill_grid, Solution): every grid point of every
field with the observed values filled in, against the oracle's full arrays, and the
reference's sol[u(t, x)] usage (src/interface/solution/timedep.jl:19-80;
test/Burgers/burgers_eq.jl:56-104 compares sol[u(t, x)] with the exact solution)."""
import math

import numpy as np
import pytest

from molgpu import Field, IV, SSPRK33, Tsit5, discretize, lower, problems, solve
from molgpu import Plan
from oracle.mol_oracle import OracleProblem

pytestmark = pytest.mark.gpu

CASES = {
    "brusselator_periodic": lambda: problems.brusselator(N=16),
    "stretched_2d_nonuniform": lambda: problems.stretched_2d(nx=14, ny=11),
    "weno_extrapolated": lambda: problems.burgers_weno_channel(nx=17, ny=13),
    "edge_robin_2d": lambda: problems.robin_2d_edge(dx=0.05, dy=0.0625),
    "adr3d": lambda: problems.adr3d(N=8, nz_pts=10),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fill_grid_matches_oracle_full_arrays(gpu_lib, name):
    s, d, _ = CASES[name]()
    spec = s.to_spec(d)
    lw = lower(spec)
    orc = OracleProblem(spec)
    plan = Plan(lw)
    v = lw.u0 + 0.02 * np.random.default_rng(2).standard_normal(lw.n_unknowns)
    for t in (0.0, 0.6):
        got = plan.fill_grid(v, t)
        ref = orc.solution_arrays(v, t, lw.param_values)
        for k, f in enumerate(lw.fields):
            assert got[k].shape == tuple(lw.npts)
            assert np.allclose(got[k], ref[f], rtol=1e-12, atol=1e-13), (name, f, t)
    plan.close()


def test_solution_saveat_ssprk33_heat(gpu_lib):
    s, d, _ = problems.heat1d(n=101)
    prob = discretize(s, d)
    sol = solve(prob, SSPRK33(), dt=2e-5, saveat=0.02)
    assert np.allclose(sol.ts, [0.0, 0.02, 0.04, 0.06, 0.08, 0.1], atol=1e-12)
    u = sol[Field("u")]
    assert u.shape == (6, 101)
    assert np.all(u[:, 0] == 0.0) and np.all(u[:, -1] == 0.0)        # Dirichlet rows
    assert np.array_equal(u[-1, 1:-1], sol.u)
    x = sol[IV("x")]
    lam = -(4 / 0.01 ** 2) * math.sin(math.pi * 0.01 / 2) ** 2
    for i, t in enumerate(sol.ts):
        assert np.max(np.abs(u[i] - math.exp(lam * t) * np.sin(math.pi * x))) < 1e-6


def test_burgers_weno_solution_on_full_grid(gpu_lib):
    """The reference's test in its own terms: sol[u(t, x)] over the whole grid (boundary and
    extrapolated points included) against x / (t + 1) at the saved times."""
    s, d, _ = problems.burgers_weno_dirichlet()
    prob = discretize(s, d)
    sol = solve(prob, Tsit5(), abstol=1e-10, reltol=1e-10, saveat=1.0)
    x = sol["x"]
    u = sol["u"]
    assert u.shape == (7, len(x))
    for i, t in enumerate(sol.ts):
        assert np.max(np.abs(u[i] - x / (t + 1))) < 1e-8, t


def test_solution_interpolation(gpu_lib):
    """sol(t, x): linear in t and x through the saved full-grid arrays (the reference's
    Gridded(Linear()) interpolation)."""
    s, d, _ = problems.heat1d(n=101)
    prob = discretize(s, d)
    sol = solve(prob, SSPRK33(), dt=2e-5, saveat=0.02)
    u = sol["u"]
    x = sol["x"]
    assert sol(0.04, x[37]) == pytest.approx(u[2, 37], rel=1e-14)
    mid = sol(0.03, 0.5 * (x[10] + x[11]))
    want = 0.25 * (u[1, 10] + u[1, 11] + u[2, 10] + u[2, 11])
    assert mid == pytest.approx(want, rel=1e-12)
    assert sol([0.0, 0.1], [0.0, 1.0]).shape == (2,)
