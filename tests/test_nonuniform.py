"""Nonuniform grids (a grid given as points, or a step that does not reach the domain's end):
per-point centered weight rows and their boundary rows, against the oracle's restatement of
CompleteCenteredDifference(d, p, x::AbstractVector) (centered_diff_weights.jl:77-153) and the
nonuniform tap selection (centered_difference.jl:32-56).  CPU only."""
import math

import numpy as np
import pytest

from desc_interp import DescInterp
from molgpu import lower, problems
from molgpu import _lib as L
from molgpu.lowering import make_axis
from molgpu.weights import centered, centered_nonuniform
from oracle.fornberg import calculate_weights, complete_centered_difference_nonuniform
from oracle.mol_oracle import OracleProblem, make_grid


def _jittered(n, seed):
    r = np.random.default_rng(seed)
    x = np.concatenate([[0.0], np.cumsum(r.uniform(0.4, 1.6, n - 1))])
    return x / x[-1]


@pytest.mark.parametrize("d", [1, 2, 3, 4])
@pytest.mark.parametrize("p", [2, 4, 6, 8])
def test_nonuniform_tables_bit_identical_to_oracle(d, p):
    for seed in (0, 1):
        x = _jittered(40, seed)
        a = centered_nonuniform(d, p, x)
        b = complete_centered_difference_nonuniform(d, p, x)
        assert a.rows == b.stencil_coefs
        assert a.low == b.low_boundary_coefs and a.high == b.high_boundary_coefs
        assert a.interior == b.stencil_coefs[0]
        assert len(a.rows) == len(x) - 2 * (a.L // 2)


@pytest.mark.parametrize("d,p", [(1, 2), (2, 2), (2, 4), (2, 8), (3, 4), (4, 6)])
def test_integer_grid_reduces_to_uniform_tables(d, p):
    """On the points 0, 1, ..., n-1 every interior row is the uniform interior row bit for
    bit (the same differences enter Fornberg's recursion) and the low rows are the uniform
    low rows; the high rows equal the uniform (mirrored) ones to rounding."""
    a = centered_nonuniform(d, p, list(range(30)))
    u = centered(d, p, 1.0)
    assert all(r == u.interior for r in a.rows)
    assert a.low == u.low
    for ra, ru in zip(a.high, u.high):
        assert np.allclose(ra, ru, rtol=0, atol=1e-11 * max(map(abs, ru)))


@pytest.mark.parametrize("d,p", [(1, 2), (1, 4), (2, 2), (2, 4), (2, 6)])
def test_rows_are_exact_on_polynomials(d, p):
    """Each row differentiates polynomials of degree below its tap count exactly (to rounding)
    at its own point: interior rows at x_i, low rows at the first nodes, high rows at the last."""
    x = _jittered(25, 3)
    op = centered_nonuniform(d, p, x)
    h = op.L // 2
    deg = op.L - 1
    c = np.random.default_rng(5).standard_normal(deg + 1)
    poly = np.polynomial.Polynomial(c)
    dpoly = poly.deriv(d)
    for k, row in enumerate(op.rows):
        i = h + k
        got = float(np.dot(row, poly(x[i - h:i + h + 1])))
        assert abs(got - dpoly(x[i])) <= 1e-7 * (1 + abs(dpoly(x[i]))), (k, got, dpoly(x[i]))
    bl = op.bLlo
    degb = bl - 1
    cb = np.random.default_rng(6).standard_normal(degb + 1)
    pb = np.polynomial.Polynomial(cb)
    dpb = pb.deriv(d)
    for k, row in enumerate(op.low):
        got = float(np.dot(row, pb(x[:bl] - x[0])))
        assert abs(got - dpb(x[k] - x[0])) <= 1e-6 * (1 + abs(dpb(x[k] - x[0])))
    n = len(x)
    for k, row in enumerate(op.high):     # high[k]: point n-1-k (0-based), nodes n-bl .. n-1
        base = x[n - 1 - bl]
        got = float(np.dot(row, pb(x[n - bl:] - base)))
        want = dpb(x[n - 1 - k] - base)
        assert abs(got - want) <= 1e-6 * (1 + abs(want))


def test_fornberg_golden_values_on_given_nodes():
    """The reference's own known answers for calculate_weights on explicit node vectors
    (test/Components/MOLfornberg_weights.jl:5-31), which the nonuniform rows are made of."""
    assert calculate_weights(2, 0.0, [-1, 0, 1.0]) == [1, -2, 1]
    assert calculate_weights(1, 0.0, [-1.0, 1.0]) == [-0.5, 0.5]
    assert calculate_weights(1, 0.0, [0, 1]) == [-1, 1]
    assert calculate_weights(1, 1.0, [0, 1]) == [-1, 1]
    assert calculate_weights(3, 0.0, [0, 1, 2, 3, 4, 5]) == [-17 / 4, 71 / 4, -59 / 2, 49 / 2, -41 / 4, 7 / 4]


def test_grid_forms():
    """An integer or a dividing step gives the uniform grid; a step that misses the end gets
    the end appended (a nonuniform grid, discretize_vars.jl:224-230); points are taken as
    given, with the end appended when missing."""
    g, dx, uni = make_axis(0.0, 1.0, 11)
    assert uni and len(g) == 11
    g, dx, uni = make_axis(0.0, 1.0, 0.03)
    assert not uni and g[-1] == 1.0 and g[-2] == pytest.approx(0.99) and len(g) == 35
    g2, _, uni2 = make_grid(0.0, 1.0, 0.03)
    assert not uni2 and np.array_equal(g, g2)
    g, _, uni = make_axis(0.0, 1.0, [0.0, 0.1, 0.5, 0.7])
    assert not uni and list(g) == [0.0, 0.1, 0.5, 0.7, 1.0]
    with pytest.raises(ValueError):
        make_axis(0.0, 1.0, [0.0, 0.5, 0.4, 1.0])


def _appended_end():
    from molgpu.api import MOLFiniteDifference
    from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, sin
    x, t = IV("x"), IV("t")
    u = Field("u")
    s = PDESystem([Eq(Differential(t)(u(x, t)), (Differential(x) ** 2)(u(x, t)))],
                  [Eq(u(x, 0.0), sin(math.pi * x)), Eq(u(0.0, t), 0.0), Eq(u(1.0, t), t)],
                  [(t, Interval(0, 1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)])
    return s.to_spec(MOLFiniteDifference({x: 0.03}, t, approx_order=4))


CASES = {
    "stretched_o2": lambda: problems.stretched_reaction_diffusion(n=41, order=2)[:2],
    "stretched_o4": lambda: problems.stretched_reaction_diffusion(n=41, order=4)[:2],
    "stretched_o6": lambda: problems.stretched_reaction_diffusion(n=41, order=6)[:2],
    "neumann_cosine_o8": lambda: problems.neumann_cosine(n=40, order=8)[:2],
    "stretched_2d": lambda: problems.stretched_2d(nx=14, ny=11)[:2],
}


def _spec(name):
    if name == "appended_end":
        return _appended_end()
    s, d = CASES[name]()
    return s.to_spec(d)


@pytest.mark.parametrize("name", sorted(CASES) + ["appended_end"])
def test_descriptor_semantics_match_oracle_nonuniform(name):
    spec = _spec(name)
    lw = lower(spec)
    orc = OracleProblem(spec)
    assert not all(lw.uniform)
    assert lw.n_unknowns == orc.n_unknowns
    assert np.array_equal(lw.u0, orc.initial_condition())
    assert any(o.rows is not None for o in lw.ops)
    di = DescInterp(lw)
    u = lw.u0 + 0.01 * np.random.default_rng(0).standard_normal(lw.n_unknowns)
    for t in (0.3, 1.5):
        a, b = orc.rhs(u, t), di.rhs(u, t)
        assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a), (name, t)


def test_neumann_cosine_tracks_exact_solution():
    """Order 8 on 40 given points: the semi-discrete RHS of cos x is -cos x to high accuracy
    (the reference's Test 03 compares the solution with exp(-t) cos x)."""
    s, d, _ = problems.neumann_cosine(n=40, order=8)
    spec = s.to_spec(d)
    orc = OracleProblem(spec)
    lw = lower(spec)
    x = lw.grids[0][lw.lower[0]:lw.npts[0] - lw.upper[0]]
    du = DescInterp(lw).rhs(np.cos(x), 0.0)
    assert np.max(np.abs(du + np.cos(x))) < 1e-6
    assert np.allclose(orc.rhs(np.cos(x), 0.0), du, rtol=0, atol=1e-12)


def test_descriptor_carries_rows():
    from molgpu import Descriptor
    s, d, _ = problems.stretched_reaction_diffusion(n=41, order=4)
    lw = lower(s.to_spec(d))
    D = Descriptor(lw)
    ops = [D.desc.ops[i] for i in range(D.desc.nops)]
    rows = [o for o in ops if o.nrows > 0]
    assert rows and all(o.nrows == lw.npts[0] - o.nlo - o.nhi for o in rows)
    o = rows[0]
    assert D.weights[o.w_int + o.L] == lw.ops[[i for i, q in enumerate(ops) if q.nrows][0]].rows[1][0]


def _unsupported(kind):
    from molgpu.api import MOLFiniteDifference, UpwindScheme
    from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, sin
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx = Differential(t), Differential(x)
    pts = problems.stretched_points(21)
    if kind == "upwind":       # second-order upwinding: the reference's table is too short
        eq, scheme = Eq(Dt(u(x, t)), -Dx(u(x, t))), UpwindScheme(2)
    else:                      # no periodic boundary on a nonuniform dimension (centered_difference.jl:36)
        eq, scheme = Eq(Dt(u(x, t)), (Dx ** 2)(u(x, t))), None
    bcs = [Eq(u(x, 0.0), sin(x))]
    bcs += [Eq(u(0.0, t), u(1.0, t))] if kind == "periodic" else [Eq(u(0.0, t), 0.0), Eq(u(1.0, t), 0.0)]
    s = PDESystem([eq], bcs, [(t, Interval(0, 1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)])
    return s.to_spec(MOLFiniteDifference({x: pts}, t, advection_scheme=scheme))


@pytest.mark.parametrize("kind", ["upwind", "periodic"])
def test_schemes_not_built_on_nonuniform_grids_are_refused(kind):
    with pytest.raises(NotImplementedError):
        lower(_unsupported(kind))


def test_plan_validation_of_rows():
    """A descriptor whose per-point rows do not match the grid fails at plan creation."""
    from molgpu import Plan
    s, d, _ = problems.stretched_reaction_diffusion(n=41, order=2)
    lw = lower(s.to_spec(d))
    op = [o for o in lw.ops if o.rows is not None][0]
    op.rows = op.rows[:-1]
    with pytest.raises(L.MolError) as e:
        Plan(lw)
    assert e.value.status == -1 and "rows" in str(e.value)


def test_generated_code_reads_the_point_row():
    """The generated interior fast path offsets the weights by the cell's own row, and the
    code compiles for sm_103a (NVRTC, no device needed)."""
    import ctypes as C
    from molgpu import Descriptor
    s, d, _ = problems.stretched_2d(nx=12, ny=9)
    D = Descriptor(lower(s.to_spec(d)))
    need = C.c_int64()
    assert L.lib().mol_generate_code(C.byref(D.desc), None, 0, C.byref(need)) == 0
    buf = C.create_string_buffer(need.value)
    assert L.lib().mol_generate_code(C.byref(D.desc), buf, need.value, C.byref(need)) == 0
    src = buf.value.decode()
    assert ".w_int + (long long)(I[0] - 2) * 3" in src
    log = C.create_string_buffer(1 << 16)
    assert L.lib().mol_codegen_compile_check(C.byref(D.desc), log, 1 << 16) == 0, log.value.decode()


UPWIND_GRIDS = ["symmetric", "left", "right", "chebyshev"]


@pytest.mark.parametrize("kind", UPWIND_GRIDS)
def test_nonuniform_upwind_tables_and_selection(kind):
    """First-order upwind tables on a nonuniform grid (upwind_diff_weights.jl:93-171) and the
    reference's selection (upwind_difference.jl:131-162): product and oracle agree bit for bit
    at every interior point, in both wind directions."""
    from molgpu.weights import select, upwind_nonuniform
    from oracle.fornberg import complete_upwind_difference_nonuniform
    from oracle.mol_oracle import upwind_taps
    x = problems.cluster_grid(kind, 41)
    n = len(x)
    for off, positive in ((0, False), (1, True)):
        a = upwind_nonuniform(1, 1, x, off)
        b = complete_upwind_difference_nonuniform(1, 1, x, off)
        assert a.rows == b.stencil_coefs and a.high == b.high_boundary_coefs
        for i in range(2, n):
            assert list(select(a, i, n, False)) == list(upwind_taps(b, i, n, False, positive)), (off, i)


def test_nonuniform_positive_wind_row_is_the_next_points():
    """Pinned reference behaviour: the operator comes back with offside 0, so the positive-wind
    difference at point i uses the row built for point i + 1 on taps i-1, i, i.e.
    (u_i - u_{i-1}) / (x_{i+1} - x_i)."""
    from molgpu.weights import select, upwind_nonuniform
    x = problems.cluster_grid("left", 21)
    op = upwind_nonuniform(1, 1, x, 1)
    for i in range(2, len(x)):
        w, taps = select(op, i, len(x), False)
        h = x[i] - x[i - 1]          # x_{i+1} - x_i in 1-based terms
        assert taps == [i - 1, i]
        assert np.allclose(w, [-1.0 / h, 1.0 / h], rtol=1e-14)


@pytest.mark.parametrize("kind", UPWIND_GRIDS)
def test_descriptor_semantics_match_oracle_nonuniform_upwind(kind):
    s, d, _ = problems.convection_nonuniform(kind, n=41)
    spec = s.to_spec(d)
    lw = lower(spec)
    orc = OracleProblem(spec)
    di = DescInterp(lw)
    u = lw.u0 + 0.01 * np.random.default_rng(0).standard_normal(lw.n_unknowns)
    for t in (0.05, 0.2):
        a, b = orc.rhs(u, t), di.rhs(u, t)
        assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a), (kind, t)


def test_nonuniform_weno_geometry_rows_reproduce_the_oracle():
    """The per-point geometry rows, evaluated as the device evaluates them, give the oracle's
    node-centred Lagrange WENO-5 (nonuniform_weno.jl:120-163) bit for bit at every target."""
    from desc_interp import _weno_nu
    from molgpu.weights import weno_nonuniform_rows, weno_nonuniform_target
    from oracle.weno_nonuniform import taps_and_target, weno_f_nonuniform
    x = _jittered(31, 7)
    rows = weno_nonuniform_rows(x)
    u = np.sin(5 * x) + 0.05 * np.random.default_rng(3).standard_normal(len(x))
    n = len(x)
    for i in range(1, n + 1):
        q0, tg = weno_nonuniform_target(i, n)
        taps, tg2 = taps_and_target(i, n)
        assert taps[0] == q0 and tg == tg2
        v = list(u[q0 - 1:q0 + 4])
        assert _weno_nu(rows[i - 1], v, 1e-6) == weno_f_nonuniform(v, 1e-6, x[q0 - 1:q0 + 4], tg), i


@pytest.mark.parametrize("kind", ["uniform", "sinh", "tanh"])
def test_descriptor_semantics_match_oracle_nonuniform_weno(kind):
    s, d, _ = problems.weno_convection_mms(kind, 41)
    spec = s.to_spec(d)
    lw = lower(spec)
    orc = OracleProblem(spec)
    assert lw.lower == [1] and lw.upper == [1]      # extent 0 on a nonuniform grid (WENO.jl:95)
    di = DescInterp(lw)
    u = lw.u0 + 0.01 * np.random.default_rng(0).standard_normal(lw.n_unknowns)
    for t in (0.01, 0.04):
        a, b = orc.rhs(u, t), di.rhs(u, t)
        assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a), (kind, t)


@pytest.mark.parametrize("kind", ["uniform", "tanh"])
def test_nonuniform_weno_converges(kind):
    """Spatial convergence of the semi-discrete operator on the manufactured solution
    (the reference's test asserts an observed order above 3.75 for the solution on the
    uniform points): the RHS error order between 81 and 161 points is above 3.5."""
    errs = []
    for n in (81, 161):
        s, d, _ = problems.weno_convection_mms(kind, n)
        spec = s.to_spec(d)
        lw = lower(spec)
        xs = lw.grids[0][1:-1]
        r = OracleProblem(spec).rhs(problems.weno_mms_exact(xs, 0.0), 0.0)
        L_ = 2 * math.pi
        exact = -(2 * math.pi / L_ * np.cos(2 * math.pi * xs / L_)
                  + problems.WENO_MMS_ALPHA * 4 * math.pi / L_ * np.cos(4 * math.pi * xs / L_))
        errs.append(np.max(np.abs(r - exact)))
    assert math.log(errs[0] / errs[1]) / math.log(2) > 3.5, errs


def test_descriptor_semantics_match_oracle_burgers_nonuniform_upwind():
    s, d, _ = problems.burgers_nonuniform_upwind()
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    u = lw.u0 + 0.01 * np.random.default_rng(0).standard_normal(lw.n_unknowns)
    a, b = orc.rhs(u, 0.3), DescInterp(lw).rhs(u, 0.3)
    assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a)


def test_chebyspace_grid():
    """chebyspace(N, x in [a, b]) (MOL_utils.jl:112-123): increasing Chebyshev points of the
    first kind with the end points set; the docs' example (100 points, Dirichlet heat) lowers
    to a nonuniform grid and matches the oracle."""
    from molgpu import IV, Interval, MOLFiniteDifference, chebyspace
    from molgpu.symbolic import Differential, Eq, Field, PDESystem, cos, exp
    x, t = IV("x"), IV("t")
    xv, pts = chebyspace(100, (x, Interval(0.0, 1.0)))
    assert xv is x and len(pts) == 100 and pts[0] == 0.0 and pts[-1] == 1.0
    assert np.all(np.diff(pts) > 0)
    k = np.arange(1, 101)
    assert np.allclose(pts[1:-1], (0.5 + 0.5 * np.cos(np.pi * (2 * k - 1) / 200))[::-1][1:-1], atol=1e-15)
    u = Field("u")
    s = PDESystem([Eq(Differential(t)(u(x, t)), (Differential(x) ** 2)(u(x, t)))],
                  [Eq(u(x, 0.0), cos(x)), Eq(u(0.0, t), exp(-1.0 * t)), Eq(u(1.0, t), exp(-1.0 * t) * math.cos(1.0))],
                  [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)])
    spec = s.to_spec(MOLFiniteDifference(dict([chebyspace(100, (x, Interval(0.0, 1.0)))]), t))
    lw = lower(spec)
    assert not lw.uniform[0] and lw.npts == [100]
    v = lw.u0 * 1.01
    a, b = OracleProblem(spec).rhs(v, 0.2), DescInterp(lw).rhs(v, 0.2)
    assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a)


# ---------------------------------------------------------------------------------------
# the nonlinear Laplacian on a nonuniform grid: per-half-point tables
# (CompleteHalfCenteredDifference(d, p, x::AbstractVector), half_offset_weights.jl:72-150),
# the outer operator on the grid's midpoints (differential_discretizer.jl:47-52)
# ---------------------------------------------------------------------------------------

@pytest.mark.parametrize("d", [0, 1, 2])
@pytest.mark.parametrize("p", [2, 4, 6])
def test_half_offset_tables_bit_identical_to_oracle(d, p):
    from molgpu.weights import half_centered_nonuniform
    from oracle.fornberg import complete_half_centered_difference_nonuniform
    for seed in (0, 1):
        x = _jittered(30, seed)
        a = half_centered_nonuniform(d, p, x)
        b = complete_half_centered_difference_nonuniform(d, p, x)
        assert a.rows == b.stencil_coefs
        assert a.low == b.low_boundary_coefs and a.high == b.high_boundary_coefs
        assert a.nlo == b.boundary_point_count and len(a.rows) == len(x) - 2 * a.nlo


@pytest.mark.parametrize("d", [0, 1, 2])
@pytest.mark.parametrize("p", [2, 4, 6])
def test_integer_grid_half_offset_reduces_to_uniform(d, p):
    """On the points 0..n-1 every interior and low row equals the uniform table bit for bit;
    the high rows (computed on the last nodes, not reflected) agree to rounding."""
    from molgpu.weights import half_centered, half_centered_nonuniform
    nu = half_centered_nonuniform(d, p, np.arange(24, dtype=float))
    un = half_centered(d, p, 1.0)
    assert all(r == un.interior for r in nu.rows)
    assert nu.low == un.low
    assert np.allclose(nu.high, un.high, rtol=0, atol=1e-13)


@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("coefficient", ["u2", "x"])
def test_descriptor_semantics_match_oracle_nonuniform_nonlinlap(order, coefficient):
    s, d, ex = problems.nonlinear_diffusion_nonuniform(order, coefficient=coefficient)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    v = lw.u0 * (1 + 0.05 * np.random.default_rng(order).standard_normal(lw.n_unknowns))
    for t in (0.0, 0.7):
        a, b = orc.rhs(v, t), DescInterp(lw).rhs(v, t)
        assert np.array_equal(a, b), (order, coefficient, t)


@pytest.mark.parametrize("order", [2, 4, 6])
def test_nonuniform_nonlinlap_is_exact_at_the_midpoints_of_midpoints(order):
    """On the reference test's exact solution (linear in x) every table is exact, so the
    semi-discrete RHS is the exact flux derivative 2 u u_x^2 taken where the outer operator
    sits: at the midpoint of the two half points around each grid point, (x[i-1] + 2x[i] +
    x[i+1])/4, not at x[i] (the outer operator is built on the grid's midpoints)."""
    s, d, ex = problems.nonlinear_diffusion_nonuniform(order)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    g = ex["points"]
    t = 0.7
    v = problems.nonlinear_diffusion_nu_exact(g[1:-1], t)
    m = (g[:-1] + g[1:]) / 2
    hm = (m[:-1] + m[1:]) / 2
    exact = 0.25 * (hm + problems.NLD_H) / (problems.NLD_C - t) ** 1.5
    for r in (orc.rhs(v, t), DescInterp(lw).rhs(v, t)):
        assert np.max(np.abs(r - exact)) <= 1e-9 * np.max(np.abs(exact))
    xi = 0.25 * (g[1:-1] + problems.NLD_H) / (problems.NLD_C - t) ** 1.5
    assert np.max(np.abs(exact - xi)) > 1e-4 * np.max(np.abs(xi))   # the offset is visible


def test_plan_validation_of_nonlinlap_rows():
    from molgpu import Plan
    s, d, _ = problems.nonlinear_diffusion_nonuniform(2)
    lw = lower(s.to_spec(d))
    term = [tm for tm in lw.terms if tm["kind"] == L.TERM_NONLINLAP][0]
    op = lw.ops[term["op"]]
    op.rows = op.rows[:-2]
    with pytest.raises(L.MolError) as e:
        Plan(lw)
    assert e.value.status == -1 and "rows" in str(e.value)


def test_generated_code_nonlinlap_rows_takes_the_runtime_tap_path():
    """With per-point rows the compile-time interior path (one row) is switched off and the
    code compiles for sm_103a (NVRTC, no device needed)."""
    import ctypes as C
    from molgpu import Descriptor
    s, d, _ = problems.nonlinear_diffusion_nonuniform(4)
    D = Descriptor(lower(s.to_spec(d)))
    need = C.c_int64()
    assert L.lib().mol_generate_code(C.byref(D.desc), None, 0, C.byref(need)) == 0
    buf = C.create_string_buffer(need.value)
    assert L.lib().mol_generate_code(C.byref(D.desc), buf, need.value, C.byref(need)) == 0
    src = buf.value.decode()
    assert src.count("if (false) {") >= 3      # forward, adjoint and face-pass fast paths
    log = C.create_string_buffer(1 << 16)
    assert L.lib().mol_codegen_compile_check(C.byref(D.desc), log, 1 << 16) == 0, log.value.decode()


# ---------------------------------------------------------------------------------------
# mixed derivatives on nonuniform grids: the product of the two per-point first-derivative rows
# ---------------------------------------------------------------------------------------

@pytest.mark.parametrize("order", [2, 4])
def test_descriptor_semantics_match_oracle_nonuniform_mixed(order):
    s, d, ex = problems.mixed_nonuniform(order=order)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    v = lw.u0 + 0.05 * np.random.default_rng(order).standard_normal(lw.n_unknowns)
    a, b = orc.rhs(v, 0.3), DescInterp(lw).rhs(v, 0.3)
    assert np.array_equal(a, b)


def test_nonuniform_mixed_is_exact_on_a_biquadratic():
    """Every order-2 row is exact on quadratics, so on u = x^2 y^2 the RHS is 2y^2 + 2x^2 +
    0.3 * 4xy at every interior point whose mixed stencil stays off the corners (the corner
    points read 0, generate_bc_eqs.jl:396-459)."""
    s, d, ex = problems.mixed_nonuniform(order=2)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    px, py = ex["points"]
    X, Y = np.meshgrid(px[1:-1], py[1:-1], indexing="ij")
    v = (X * X * Y * Y).reshape(-1, order="F")
    exact = (2 * Y * Y + 2 * X * X + 1.2 * X * Y)
    for r in (orc.rhs(v, 0.0), DescInterp(lw).rhs(v, 0.0)):
        R = r.reshape(X.shape, order="F")
        assert np.max(np.abs(R[1:-1, 1:-1] - exact[1:-1, 1:-1])) <= 1e-9 * np.max(np.abs(exact))


def test_generated_code_mixed_rows_takes_the_runtime_tap_path():
    import ctypes as C
    from molgpu import Descriptor
    s, d, _ = problems.mixed_nonuniform(nx=11, ny=9)
    D = Descriptor(lower(s.to_spec(d)))
    need = C.c_int64()
    assert L.lib().mol_generate_code(C.byref(D.desc), None, 0, C.byref(need)) == 0
    buf = C.create_string_buffer(need.value)
    assert L.lib().mol_generate_code(C.byref(D.desc), buf, need.value, C.byref(need)) == 0
    assert buf.value.decode().count("if (false) {") >= 2
    log = C.create_string_buffer(1 << 16)
    assert L.lib().mol_codegen_compile_check(C.byref(D.desc), log, 1 << 16) == 0, log.value.decode()
