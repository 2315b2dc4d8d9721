"""The spherical Laplacian rule (spherical_laplacian.jl:10-130) on the GPU: the right-hand side
and fixed SSPRK33 steps of the forms the lowering rewrites, on a uniform r grid and on a grid
given as points, against the oracle's restatement."""
import math

import numpy as np
import pytest

from molgpu import Plan, lower, problems
from molgpu.api import MOLFiniteDifference
from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, exp, sin
from oracle.integrators import ssprk33
from oracle.mol_oracle import OracleProblem

pytestmark = pytest.mark.gpu

FORMS = {
    "one_over_r2_times": lambda r, u, Dr: 1.0 / r ** 2 * Dr(r ** 2 * Dr(u)),
    "state_coefficient": lambda r, u, Dr: Dr(r ** 2 * (1.0 + u) * Dr(u)) / r ** 2,
    "coordinate_coefficient": lambda r, u, Dr: 1.0 / r ** 2 * Dr((2.0 + r) * r ** 2 * Dr(u)),
}


def _spec(form, grid, order):
    r, t = IV("r"), IV("t")
    u = Field("u")
    Dt, Dr = Differential(t), Differential(r)
    bcs = [Eq(u(r, 0.0), sin(r) / r), Eq(Dr(u(0.0, t)), 0.0), Eq(u(1.0, t), exp(-t) * math.sin(1.0))]
    s = PDESystem([Eq(Dt(u(r, t)), FORMS[form](r, u(r, t), Dr))], bcs,
                  [(t, Interval(0, 1)), (r, Interval(0.0, 1.0))], [t, r], [u(r, t)])
    return s.to_spec(MOLFiniteDifference({r: grid}, t, approx_order=order))


@pytest.mark.parametrize("grid", ["uniform", "points"])
@pytest.mark.parametrize("order", [2, 4])
@pytest.mark.parametrize("form", sorted(FORMS))
def test_spherical_rule_on_gpu(gpu_lib, form, order, grid):
    g = 0.05 if grid == "uniform" else problems.stretched_points(31)
    spec = _spec(form, g, order)
    lw, orc = lower(spec), OracleProblem(spec)
    plan = Plan(lw)
    v = lw.u0 * (1 + 0.05 * np.random.default_rng(order).standard_normal(lw.n_unknowns))
    for t in (0.0, 0.4):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, v, None, t)
        ref = orc.rhs(v, t)
        assert np.linalg.norm(du - ref) <= 1e-12 * np.linalg.norm(ref), (form, order, grid, t)
    dr = float(np.min(np.diff(lw.grids[0])))
    dt = 0.02 * dr * dr          # explicit stability with the coefficient up to 3 and the 1/r term
    u = lw.u0.copy()
    plan.step_ssprk33(u, dt, 20)
    ref, _ = ssprk33(lambda w, tt: orc.rhs(w, tt), lw.u0, 0.0, dt, 20)
    assert np.linalg.norm(u - ref) <= 1e-10 * np.linalg.norm(ref)
    plan.close()
