"""The oracle's upwind and WENO rows against the reference's 1-D linear convection tests (no
device needed).

``test/Convection/MOL_1D_Linear_Convection.jl`` (first-order upwinding, explicit Euler at
dt = dx) and ``test/Convection_WENO/MOL_1D_Linear_Convection_WENO.jl`` (WENO5, SSPRK33 at
dt = 0.01) carry a Gaussian once around the periodic interval [0, 2] and compare sol[u] at
t = 2 (grid points 2..end) with the initial profile, in the 2-norm within atol 0.1 (Julia's
isapprox on arrays).  The same systems are built with the front end and stepped through the
oracle's right-hand side with the reference's integrator and step.
"""
import math

import numpy as np
import pytest

from molgpu.api import MOLFiniteDifference, WENOScheme
from molgpu.symbolic import Differential, Eq, Field, Interval, IV, Param, PDESystem, exp
from oracle.integrators import ssprk33
from oracle.mol_oracle import OracleProblem

DX = 2 / 80


def _asf(x):
    return (0.5 / (0.2 * math.sqrt(2.0 * 3.1415))) * exp(-(x - 1.0) ** 2 / (2.0 * 0.2 ** 2))


def _problem(rhs_of, weno, with_param=False):
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dx = Differential(x)
    params = [Param("v", 1.0)] if with_param else []
    eq = Eq(Differential(t)(u(x, t)), rhs_of(u(x, t), Dx, params))
    sys_ = PDESystem([eq], [Eq(u(x, 0.0), _asf(x)), Eq(u(0.0, t), u(2.0, t))],
                     [(t, Interval(0.0, 2.0)), (x, Interval(0.0, 2.0))], [t, x], [u(x, t)], params)
    kw = {"advection_scheme": WENOScheme()} if weno else {}
    return OracleProblem(sys_.to_spec(MOLFiniteDifference({x: DX}, t, **kw)))


def _euler(orc, dt, nsteps):
    u = orc.initial_condition()
    for k in range(nsteps):
        u = u + dt * orc.rhs(u, k * dt)
    return u


def _error_at_2(orc, u):
    full = orc.solution_arrays(u, 2.0, orc.param_values)["u"]
    xs = orc.grid[0][1:]
    want = (0.5 / (0.2 * math.sqrt(2.0 * 3.1415))) * np.exp(-(xs - 1.0) ** 2 / (2.0 * 0.2 ** 2))
    return float(np.linalg.norm(full[1:] - want))


CASES = {
    "00: u_t = -u_x": (lambda U, Dx, p: -1.0 * Dx(U), False),
    "00a: u_t = u_x": (lambda U, Dx, p: Dx(U), False),
    "02: u_t = -v u_x": (lambda U, Dx, p: -1.0 * p[0] * Dx(U), True),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_upwind_convection(name):
    """MOL_1D_Linear_Convection.jl:9-58, 59-108, 257-315: Euler at dt = 0.025 to t = 2."""
    rhs_of, with_param = CASES[name]
    orc = _problem(rhs_of, weno=False, with_param=with_param)
    assert _error_at_2(orc, _euler(orc, 0.025, 80)) <= 0.1


@pytest.mark.parametrize("name", sorted(CASES))
def test_weno_convection(name):
    """MOL_1D_Linear_Convection_WENO.jl:10-58, 59-107, 257-316: SSPRK33 at dt = 0.01 to t = 2."""
    rhs_of, with_param = CASES[name]
    orc = _problem(rhs_of, weno=True, with_param=with_param)
    u, _ = ssprk33(lambda v, s: orc.rhs(v, s), orc.initial_condition(), 0.0, 0.01, 200)
    assert _error_at_2(orc, u) <= 0.1
