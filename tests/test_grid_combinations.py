"""Combinations of the grid and boundary variants in 2-D and 3-D, lowered and evaluated with
the kernels' semantics on the CPU against the oracle (the GPU tests cover each variant)."""
import math

import numpy as np
import pytest

from desc_interp import DescInterp
from molgpu import lower, problems
from molgpu.api import MOLFiniteDifference, UpwindScheme, WENOScheme
from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, cos, sin
from oracle.mol_oracle import OracleProblem


def _weno_nonuniform_x_periodic_y():
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    Dt, Dx, Dy = Differential(t), Differential(x), Differential(y)
    eq = Eq(Dt(u(x, y, t)), -u(x, y, t) * Dx(u(x, y, t)) - 0.4 * Dy(u(x, y, t)) + 0.01 * (Dy ** 2)(u(x, y, t)))
    bcs = [Eq(u(x, y, 0.0), 0.6 + 0.2 * sin(3.0 * x) * cos(2.0 * math.pi * y)),
           Eq(u(0.0, y, t), 0.6), Eq(u(1.0, y, t), 0.6 + 0.1 * t), Eq(u(x, 0.0, t), u(x, 1.0, t))]
    s = PDESystem([eq], bcs, [(t, Interval(0, 1)), (x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0))], [t, x, y],
                  [u(x, y, t)])
    return s.to_spec(MOLFiniteDifference({x: problems.stretched_points(23), y: 17}, t,
                                         advection_scheme=WENOScheme()))


def _nonuniform_3d():
    x, y, z, t = IV("x"), IV("y"), IV("z"), IV("t")
    u = Field("u")
    Dt = Differential(t)
    lap = (Differential(x) ** 2)(u(x, y, z, t)) + (Differential(y) ** 2)(u(x, y, z, t)) + \
        (Differential(z) ** 2)(u(x, y, z, t))
    eq = Eq(Dt(u(x, y, z, t)), lap - 0.5 * Differential(z)(u(x, y, z, t)))
    bcs = [Eq(u(x, y, z, 0.0), 1.0 + 0.1 * x * y * z)]
    for v in (x, y, z):
        for end in (0.0, 1.0):
            args = [x, y, z]
            args[[x, y, z].index(v)] = end
            bcs.append(Eq(u(*args, t), 1.0))
    s = PDESystem([eq], bcs, [(t, Interval(0, 1)), (x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0)),
                              (z, Interval(0.0, 1.0))], [t, x, y, z], [u(x, y, z, t)])
    return s.to_spec(MOLFiniteDifference({x: 9, y: problems.stretched_points(8), z: problems.cluster_grid("left", 10)},
                                         t, approx_order=4))


def _edge_upwind_2d():
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    Dt, Dx, Dy = Differential(t), Differential(x), Differential(y)
    eq = Eq(Dt(u(x, y, t)), (Dx ** 2)(u(x, y, t)) + (Dy ** 2)(u(x, y, t)) - 0.7 * Dx(u(x, y, t)) + 0.3 * Dy(u(x, y, t)))
    bcs = [Eq(u(x, y, 0.0), 1.0 + 0.2 * cos(3.0 * x) * sin(2.0 * y)), Eq(u(0.0, y, t), 1.0),
           Eq(Dx(u(1.0, y, t)), 0.0), Eq(u(x, 0.0, t) + 0.5 * Dy(u(x, 0.0, t)), 1.0 + t), Eq(u(x, 1.0, t), 1.0)]
    s = PDESystem([eq], bcs, [(t, Interval(0, 1)), (x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0))], [t, x, y],
                  [u(x, y, t)])
    return s.to_spec(MOLFiniteDifference({x: 0.1, y: 0.125}, t, approx_order=4, grid_align="edge",
                                         advection_scheme=UpwindScheme(2)))


def _two_fields_nonuniform():
    x, t = IV("x"), IV("t")
    u, v = Field("u"), Field("v")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    eqs = [Eq(Dt(u(x, t)), Dxx(u(x, t)) - u(x, t) * v(x, t)), Eq(Dt(v(x, t)), 0.5 * Dxx(v(x, t)) + u(x, t))]
    bcs = [Eq(u(x, 0.0), sin(math.pi * x)), Eq(v(x, 0.0), 1.0 + 0.0 * x), Eq(u(0.0, t), 0.0), Eq(u(1.0, t), 0.0),
           Eq(Dx(v(0.0, t)), 0.0), Eq(v(1.0, t) + Dx(v(1.0, t)), 1.0)]
    s = PDESystem(eqs, bcs, [(t, Interval(0, 1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t), v(x, t)])
    return s.to_spec(MOLFiniteDifference({x: problems.cluster_grid("chebyshev", 31)}, t, approx_order=6))


CASES = {"weno_nonuniform_x_periodic_y": _weno_nonuniform_x_periodic_y, "nonuniform_3d": _nonuniform_3d,
         "edge_upwind_2d": _edge_upwind_2d, "two_fields_nonuniform": _two_fields_nonuniform}


@pytest.mark.parametrize("name", sorted(CASES))
def test_combination_matches_oracle(name):
    spec = CASES[name]()
    lw = lower(spec)
    orc = OracleProblem(spec)
    assert lw.n_unknowns == orc.n_unknowns
    assert np.array_equal(lw.u0, orc.initial_condition())
    u = lw.u0 + 0.01 * np.random.default_rng(1).standard_normal(lw.n_unknowns)
    for t in (0.1, 0.7):
        a, b = orc.rhs(u, t), DescInterp(lw).rhs(u, t)
        assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a), (name, t)
