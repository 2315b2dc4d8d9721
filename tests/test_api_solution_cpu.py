"""The host side of solve/Solution (save times, stepping segments, sol[u], sol[x], sol(t, x)),
checked on the CPU with a stand-in plan that steps with the oracle."""
import math

import numpy as np
import pytest

from molgpu import Field, IV, SSPRK33, Tsit5, lower, problems
from molgpu.api import ODEProblem, Solution, solve
from oracle.integrators import ssprk33, tsit5
from oracle.mol_oracle import OracleProblem


class OraclePlan:
    """Implements the three Plan calls solve/Solution use, with the oracle."""

    def __init__(self, lw, spec):
        self.lowered = lw
        self.orc = OracleProblem(spec)
        self.calls = []

    def step_ssprk33(self, u, dt, n, t0=0.0, p=None):
        self.calls.append(("ssprk33", t0, n))
        u[:], _ = ssprk33(lambda v, t: self.orc.rhs(v, t), u.copy(), t0, dt, n)

    def solve_tsit5(self, u, t0, t1, abstol, reltol, p=None, dt0=0.0):
        self.calls.append(("tsit5", t0, t1))
        out, st = tsit5(lambda v, t: self.orc.rhs(v, t), u.copy(), t0, t1, abstol, reltol)
        u[:] = out
        return st

    def fill_grid(self, u, t, p=None):
        full = self.orc.solution_arrays(u, t, self.lowered.param_values)
        return np.stack([full[f] for f in self.lowered.fields])


class FakeF:
    def __init__(self, plan):
        self.plan = plan


def _prob(n=21):
    s, d, _ = problems.heat1d(n=n)
    spec = s.to_spec(d)
    lw = lower(spec)
    plan = OraclePlan(lw, spec)
    return ODEProblem(FakeF(plan), lw.u0.copy(), (0.0, 0.1), lw.param_values.copy(), lw), plan


def test_saveat_step_splits_the_fixed_step_run():
    prob, plan = _prob()
    sol = solve(prob, SSPRK33(), dt=1e-4, saveat=0.025)
    assert np.allclose(sol.ts, [0.0, 0.025, 0.05, 0.075, 0.1])
    assert [c[2] for c in plan.calls] == [250, 250, 250, 250]
    whole, _ = ssprk33(lambda v, t: plan.orc.rhs(v, t), prob.u0.copy(), 0.0, 1e-4, 1000)
    assert np.allclose(sol.u, whole, rtol=1e-13, atol=1e-15)
    with pytest.raises(ValueError):
        solve(prob, SSPRK33(), dt=3e-4, saveat=[0.05])      # not on the step grid


def test_solution_indexing_and_interpolation():
    prob, plan = _prob()
    sol = solve(prob, SSPRK33(), dt=1e-4, saveat=[0.05, 0.1])
    u = sol[Field("u")]
    x = sol[IV("x")]
    assert u.shape == (3, 21) and np.array_equal(sol["u"], u)
    assert np.all(u[:, 0] == 0.0) and np.all(u[:, -1] == 0.0)
    assert np.array_equal(u[-1, 1:-1], sol.u)
    assert sol(0.05, x[7]) == pytest.approx(u[1, 7], rel=1e-14)
    assert sol(0.075, x[7]) == pytest.approx(0.5 * (u[1, 7] + u[2, 7]), rel=1e-13)
    assert set(sol.grid) == {"x"}


def test_tsit5_segments_meet_the_save_times():
    prob, plan = _prob()
    sol = solve(prob, Tsit5(), abstol=1e-10, reltol=1e-10, saveat=0.05)
    assert [c[1:] for c in plan.calls] == [(0.0, 0.05), (0.05, 0.1)]
    assert np.allclose(sol.ts, [0.0, 0.05, 0.1])
    lam = -(4 / 0.05 ** 2) * math.sin(math.pi * 0.05 / 2) ** 2
    xs = prob.lowered.grids[0][1:-1]
    assert np.max(np.abs(sol.u - math.exp(lam * 0.1) * np.sin(math.pi * xs))) < 1e-8
