"""The spherical Laplacian r^-2 Dr(c r^2 Dr(u)) through the reference's spherical_diffusion
rule (src/discretization/schemes/spherical_laplacian/spherical_laplacian.jl:10-130): the
lowering against the oracle's independent restatement, and the rule's value on data every
table is exact for.  CPU only."""
import math

import numpy as np
import pytest

from desc_interp import DescInterp
from molgpu import lower, problems
from molgpu.api import MOLFiniteDifference
from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, exp, sin
from oracle.integrators import tsit5
from oracle.mol_oracle import OracleProblem


def _system(rhs, bcs=None, dr=0.1, order=4):
    r, t = IV("r"), IV("t")
    u = Field("u")
    Dt, Dr = Differential(t), Differential(r)
    if bcs is None:
        bcs = [Eq(u(r, 0.0), sin(r) / r), Eq(Dr(u(0.0, t)), 0.0), Eq(u(1.0, t), exp(-t) * math.sin(1.0))]
    s = PDESystem([Eq(Dt(u(r, t)), rhs(r, u(r, t), Dr))], bcs, [(t, Interval(0, 1)), (r, Interval(0.0, 1.0))],
                  [t, r], [u(r, t)])
    return s.to_spec(MOLFiniteDifference({r: dr}, t, approx_order=order))


FORMS = {
    "one_over_r2_times": lambda r, u, Dr: 1.0 / r ** 2 * Dr(r ** 2 * Dr(u)),
    "divided_by_r2": lambda r, u, Dr: Dr(r ** 2 * Dr(u)) / r ** 2,
    "scaled": lambda r, u, Dr: 4.0 / r ** 2 * Dr(r ** 2 * Dr(u)),
    "state_coefficient": lambda r, u, Dr: Dr(r ** 2 * (1.0 + u) * Dr(u)) / r ** 2,
    "coordinate_coefficient": lambda r, u, Dr: 1.0 / r ** 2 * Dr((2.0 + r) * r ** 2 * Dr(u)),
}


@pytest.mark.parametrize("order", [2, 4])
@pytest.mark.parametrize("form", sorted(FORMS))
def test_spherical_rule_matches_oracle(form, order):
    spec = _system(FORMS[form], order=order)
    lw, orc = lower(spec), OracleProblem(spec)
    v = lw.u0 * (1 + 0.05 * np.random.default_rng(order).standard_normal(lw.n_unknowns))
    for t in (0.0, 0.4):
        a, b = orc.rhs(v, t), DescInterp(lw).rhs(v, t)
        assert np.array_equal(a, b), (form, order, t)


def test_spherical_rule_value_on_a_quadratic():
    """On u = r^2 (Dr(u) = 0 at r = 0, u = 1 at r = 1) every order-2 table is exact, so the rule
    as the reference writes it, D1(u)/r + Dr(Dr(u)), is 2 + 2 = 4 at every unknown; the
    operator r^-2 (r^2 u_r)_r itself is 6 there, and the plain nonlinear Laplacian of r^2
    followed by the 1/r^2 factor (what the expression is without the rule) is neither."""
    r, t = IV("r"), IV("t")
    u = Field("u")
    Dr = Differential(r)
    bcs = [Eq(u(r, 0.0), r * r), Eq(Dr(u(0.0, t)), 0.0), Eq(u(1.0, t), 1.0)]
    spec = _system(FORMS["one_over_r2_times"], bcs=bcs, dr=0.05, order=2)
    lw, orc = lower(spec), OracleProblem(spec)
    g = lw.grids[0][1:-1]
    for rhs in (orc.rhs(g * g, 0.0), DescInterp(lw).rhs(g * g, 0.0)):
        assert np.allclose(rhs, 4.0, rtol=0, atol=1e-10)


@pytest.mark.parametrize("scale,order", [(1.0, 4), (4.0, 2)])
def test_reference_tests_07_and_08_bars(scale, order):
    """The reference's Tests 07 (order 4) and 08 (scale 4, order 2) hold every unknown within
    0.06 of e^(-scale t) sin(r)/r at the save times 0.1, ..., 1 (dr = 0.1).  The restated rule
    integrated with Tsit5 stays inside by a small margin (0.0555 at worst), where the
    continuous operator's error would be near 1e-5: the bar was set for this scheme."""
    s, d, ex = problems.spherical_laplacian(dr=0.1, order=order, scale=scale)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    g = lw.grids[0][1:-1]
    u = lw.u0.copy()
    worst = 0.0
    for k in range(10):
        u, _ = tsit5(lambda w, tt: orc.rhs(w, tt), u, 0.1 * k, 0.1 * (k + 1), 1e-8, 1e-8)
        worst = max(worst, float(np.max(np.abs(u - math.exp(-scale * 0.1 * (k + 1)) * np.sin(g) / g))))
    assert 0.05 < worst < 0.06


def test_spherical_rule_with_r0_as_an_unknown_is_refused():
    r, t = IV("r"), IV("t")
    u = Field("u")
    Dt, Dr = Differential(t), Differential(r)
    s = PDESystem([Eq(Dt(u(r, t)), Dr(r ** 2 * Dr(u(r, t))) / r ** 2)],
                  [Eq(u(r, 0.0), 1.0 + 0.0 * r), Eq(u(-1.0, t), 1.0), Eq(u(1.0, t), 1.0)],
                  [(t, Interval(0, 1)), (r, Interval(-1.0, 1.0))], [t, r], [u(r, t)])
    with pytest.raises(NotImplementedError):
        lower(s.to_spec(MOLFiniteDifference({r: 0.1}, t)))


@pytest.mark.parametrize("order", [2, 4])
def test_spherical_rule_on_a_nonuniform_grid(order):
    """On a grid given as points the rule's first derivative and nonlinear Laplacian use the
    per-point tables (centered_difference.jl:32-56, half_offset_weights.jl:72-150)."""
    r, t = IV("r"), IV("t")
    u = Field("u")
    Dt, Dr = Differential(t), Differential(r)
    s = PDESystem([Eq(Dt(u(r, t)), Dr(r ** 2 * (1.0 + u(r, t)) * Dr(u(r, t))) / r ** 2)],
                  [Eq(u(r, 0.0), sin(r) / r), Eq(Dr(u(0.0, t)), 0.0), Eq(u(1.0, t), exp(-t) * math.sin(1.0))],
                  [(t, Interval(0, 1)), (r, Interval(0.0, 1.0))], [t, r], [u(r, t)])
    spec = s.to_spec(MOLFiniteDifference({r: problems.stretched_points(31)}, t, approx_order=order))
    lw, orc = lower(spec), OracleProblem(spec)
    assert any(o.rows is not None for o in lw.ops)
    v = lw.u0 * 1.01
    assert np.array_equal(orc.rhs(v, 0.3), DescInterp(lw).rhs(v, 0.3))
