"""WENO along a bounded (non-periodic) uniform dimension: the interior stops two points from
each end (WENO.jl:94, interior_map.jl:117-139) and points 2 and n-1 are observed through the
extrapolation rows of BoundaryInterpolatorExtrapolator(max(6, order), dx)
(generate_extrap_eqs!, generate_bc_eqs.jl:336-392; extrapolation_weights.jl:1-60).  CPU only."""
from fractions import Fraction

import numpy as np
import pytest

from desc_interp import DescInterp
from molgpu import lower, problems
from molgpu import _lib as L
from molgpu.weights import extrapolator
from oracle.fornberg import boundary_interpolator_extrapolator
from oracle.mol_oracle import OracleProblem


def _lagrange(x0, nodes):
    out = []
    for k in nodes:
        v = Fraction(1)
        for m in nodes:
            if m != k:
                v *= Fraction(x0 - m, k - m)
        out.append(v)
    return out


@pytest.mark.parametrize("q", [6, 7, 8, 10])
def test_extrapolator_tables(q):
    """Product and oracle tables agree bit for bit, and every low row is the Lagrange
    interpolation of its node from the other q - 1 nodes, a zero in its own slot (exact
    rationals, rounded once)."""
    a = extrapolator(q)
    b = boundary_interpolator_extrapolator(q, 0.05)
    assert a.low == b.low_boundary_coefs and a.high == b.high_boundary_coefs
    assert a.interior == b.stencil_coefs
    for x0, row in enumerate(a.low):
        nodes = [m for m in range(q) if m != x0]
        exact = _lagrange(x0, nodes)
        got = row[:x0] + row[x0 + 1:]
        assert row[x0] == 0.0
        assert np.allclose(got, [float(e) for e in exact], rtol=1e-13, atol=1e-13)
    assert a.high[1] == a.low[1][::-1]


CASES = {
    "inviscid_dirichlet": lambda: problems.burgers_weno_dirichlet(),
    "viscous_o2": lambda: problems.viscous_burgers_weno_bounded(n=33, order=2),
    "viscous_o8": lambda: problems.viscous_burgers_weno_bounded(n=33, order=8),
    "channel_2d": lambda: problems.burgers_weno_channel(nx=17, ny=13),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_descriptor_semantics_match_oracle_weno_bounded(name):
    s, d, _ = CASES[name]()
    spec = s.to_spec(d)
    lw = lower(spec)
    orc = OracleProblem(spec)
    assert lw.lower[0] == 2 and lw.upper[0] == 2
    assert lw.n_unknowns == orc.n_unknowns
    assert np.array_equal(lw.u0, orc.initial_condition())
    assert all(e["extrap"] > 0 for (f, j, side), e in lw.bcs.items() if j == 0)
    di = DescInterp(lw)
    u = lw.u0 + 0.01 * np.random.default_rng(0).standard_normal(lw.n_unknowns)
    for t in (0.3, 1.5):
        a, b = orc.rhs(u, t), di.rhs(u, t)
        assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a), (name, t)


def test_linear_solution_is_reproduced_exactly():
    """u = x / (t + 1) solves u_t = -u u_x; WENO and the extrapolation rows are exact on
    linear data, so the semi-discrete RHS equals -x / (t + 1)^2 to rounding (the reference's
    test/Burgers/burgers_eq.jl:56-104 checks the solution against it)."""
    s, d, _ = problems.burgers_weno_dirichlet()
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    x = lw.grids[0][2:-2]
    for t in (0.0, 2.5):
        for r in (orc.rhs(x / (t + 1), t), DescInterp(lw).rhs(x / (t + 1), t)):
            assert np.max(np.abs(r + x / (t + 1) ** 2)) < 1e-13


def _variant(kind):
    from molgpu.api import MOLFiniteDifference, WENOScheme
    from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, sin
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dx = Differential(x)
    bcs = [Eq(u(x, 0.0), sin(x))]
    if kind == "neumann":
        bcs += [Eq(Dx(u(0.0, t)), 0.0), Eq(u(1.0, t), 0.0)]
    elif kind == "missing":
        bcs += [Eq(u(0.0, t), 0.0)]
    s = PDESystem([Eq(Differential(t)(u(x, t)), -u(x, t) * Dx(u(x, t)))], bcs,
                  [(t, Interval(0, 1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)])
    return s.to_spec(MOLFiniteDifference({x: 0.05}, t, advection_scheme=WENOScheme()))


@pytest.mark.parametrize("kind", ["neumann", "missing"])
def test_coupled_extrapolation_cases_refused(kind):
    """Next to a Neumann/Robin row, or with no row at an end, the extrapolated point and the
    boundary point depend on each other (the reference solves the pair symbolically); those
    forms are refused with NotImplementedError."""
    with pytest.raises(NotImplementedError):
        lower(_variant(kind))


def test_plan_refuses_weno_bounded_without_extrapolation_rows():
    from molgpu import Plan
    s, d, _ = problems.burgers_weno_dirichlet()
    lw = lower(s.to_spec(d))
    for e in lw.bcs.values():
        e["extrap"] = 0
    with pytest.raises(L.MolError) as e:
        Plan(lw)
    assert e.value.status == -6
