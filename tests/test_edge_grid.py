"""Edge-aligned grids (grid_align = edge_align): cell centres plus one ghost point beyond each
end (discretize_vars.jl:373-390), boundary rows at the faces through the half-offset
interpolation and derivative tables solved for the ghost point (boundary_value_maps for
EdgeAlignedGrid, generate_bc_eqs.jl:80-160).  CPU only."""
import math

import numpy as np
import pytest

from desc_interp import DescInterp
from molgpu import lower, problems
from molgpu import _lib as L
from molgpu.lowering import make_edge_axis
from oracle.mol_oracle import OracleProblem, make_edge_grid


def test_edge_grid_points():
    g, dx, _ = make_edge_axis(0.0, 1.0, 0.05)
    assert len(g) == 22 and g[0] == -0.025 and g[1] == 0.025 and g[-1] == 1.025
    assert np.array_equal(g, make_edge_grid(0.0, 1.0, 0.05)[0])
    g, dx, _ = make_edge_axis(0.0, 1.0, 20)       # an integer is a number of cells
    assert dx == 0.05 and len(g) == 22
    with pytest.raises(NotImplementedError):       # the step misses the end: a grid of midpoints
        make_edge_axis(0.0, 1.0, 0.03)


CASES = {
    "neumann_o2": lambda: problems.neumann_cosine_edge(dx=0.05, order=2),
    "neumann_o4": lambda: problems.neumann_cosine_edge(dx=0.05, order=4),
    "neumann_o8": lambda: problems.neumann_cosine_edge(dx=0.01, order=8),
    "robin_2d": lambda: problems.robin_2d_edge(dx=0.05, dy=0.0625),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_descriptor_semantics_match_oracle_edge(name):
    s, d, _ = CASES[name]()
    spec = s.to_spec(d)
    lw = lower(spec)
    orc = OracleProblem(spec)
    assert lw.n_unknowns == orc.n_unknowns
    assert np.array_equal(lw.u0, orc.initial_condition())
    assert all(e["kind"] == L.BC_EDGE for e in lw.bcs.values())
    di = DescInterp(lw)
    u = lw.u0 + 0.01 * np.random.default_rng(0).standard_normal(lw.n_unknowns)
    for t in (0.3, 1.5):
        a, b = orc.rhs(u, t), di.rhs(u, t)
        assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a), (name, t)


@pytest.mark.parametrize("order,dx,tol", [(2, 0.05, 0.03), (4, 0.05, 1e-3), (8, 0.01, 1e-9)])
def test_edge_neumann_rhs_converges(order, dx, tol):
    """cos(pi x) satisfies u_x = 0 at both faces: the semi-discrete RHS approximates
    -pi^2 cos(pi x) at the cell centres to the scheme's order."""
    s, d, _ = problems.neumann_cosine_edge(dx=dx, order=order)
    spec = s.to_spec(d)
    lw = lower(spec)
    xs = lw.grids[0][1:-1]
    r = OracleProblem(spec).rhs(np.cos(math.pi * xs), 0.0)
    assert np.max(np.abs(r + math.pi ** 2 * np.cos(math.pi * xs))) < tol


def test_edge_combinations_not_built_are_refused():
    from molgpu.api import MOLFiniteDifference, WENOScheme
    from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, sin
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dx = Differential(x)
    dom = [(t, Interval(0, 1)), (x, Interval(0.0, 1.0))]
    per = PDESystem([Eq(Differential(t)(u(x, t)), (Dx ** 2)(u(x, t)))],
                    [Eq(u(x, 0.0), sin(x)), Eq(u(0.0, t), u(1.0, t))], dom, [t, x], [u(x, t)])
    with pytest.raises(NotImplementedError):
        lower(per.to_spec(MOLFiniteDifference({x: 0.05}, t, grid_align="edge")))
    weno = PDESystem([Eq(Differential(t)(u(x, t)), -u(x, t) * Dx(u(x, t)))],
                     [Eq(u(x, 0.0), sin(x)), Eq(u(0.0, t), 0.0), Eq(u(1.0, t), 0.0)], dom, [t, x], [u(x, t)])
    with pytest.raises(NotImplementedError):
        lower(weno.to_spec(MOLFiniteDifference({x: 0.05}, t, grid_align="edge", advection_scheme=WENOScheme())))
