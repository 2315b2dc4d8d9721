"""Host-side logic on the CPU: weights, lowering, descriptor semantics, C-ABI exports."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from desc_interp import DescInterp
from molgpu import _lib as L
from molgpu import lower, problems, weights
from oracle import fornberg as OF
from oracle.mol_oracle import OracleProblem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("d,p", [(1, 2), (2, 2), (3, 2), (4, 2), (1, 4), (2, 4), (2, 6), (1, 3)])
@pytest.mark.parametrize("dx", [1.0, 0.01, 1 / 256, 2 * np.pi / 65536, 1 / 257, 0.3])
def test_product_tables_bit_identical_to_oracle(d, p, dx):
    a = weights.centered(d, p, dx)
    b = OF.complete_centered_difference(d, p, dx)
    assert a.interior == b.stencil_coefs
    assert a.low == b.low_boundary_coefs and a.high == b.high_boundary_coefs
    for off in (0, d + p - 1):
        a = weights.upwind(d, p, dx, off)
        b = OF.complete_upwind_difference(d, p, dx, off)
        assert a.interior == b.stencil_coefs
        assert a.low == b.low_boundary_coefs and a.high == b.high_boundary_coefs
    a = weights.half_centered(d % 2, p, dx)
    b = OF.complete_half_centered_difference(d % 2, p, dx)
    assert a.interior == b.stencil_coefs and a.low == b.low_boundary_coefs


def test_fornberg_product_golden():
    import json
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_known_answers.json")))
    for c in g["fornberg"]:
        assert weights.fornberg(c["order"], c["x0"], c["x"]) == c["expected"]


SMALL = [
    ("heat1d", dict(n=11)), ("brusselator", dict(N=8)), ("burgers", dict(npts=33)),
    ("nonlinear_diffusion", dict(n=9, k=1.3, seed=1000)), ("nonlinear_diffusion", dict(n=5, k=0.2, seed=1005)),
    ("adr3d", dict(N=6, nz_pts=8)),
]


@pytest.mark.parametrize("name,kw", SMALL)
def test_descriptor_semantics_match_oracle(name, kw):
    """The lowered descriptor, evaluated with the kernels' semantics on the CPU, equals the oracle."""
    sys_, disc, _ = getattr(problems, name)(**kw)
    spec = sys_.to_spec(disc)
    lw = lower(spec)
    orc = OracleProblem(spec)
    assert lw.n_unknowns == orc.n_unknowns
    assert np.array_equal(lw.u0, orc.initial_condition())
    di = DescInterp(lw)
    u = lw.u0 + 0.01 * np.random.default_rng(0).standard_normal(lw.n_unknowns)
    for t in (0.3, 1.5):
        a, b = orc.rhs(u, t), di.rhs(u, t)
        assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a)


def test_unknown_layout_matches_generated_code():
    """Brusselator dx=1/4: u[2,2], u[3,2], ... then v[...] (docs/src/generated/bruss_code.md)."""
    sys_, disc, _ = problems.brusselator(N=4)
    lw = lower(sys_.to_spec(disc))
    assert lw.npts == [5, 5] and lw.lower == [1, 1] and lw.upper == [0, 0]
    assert lw.n_unknowns == 32
    # first unknowns walk x fastest starting at grid index 2
    x = lw.interior_coords()["x"].reshape(-1, order="F")
    assert list(x[:4]) == [0.25, 0.5, 0.75, 1.0]


def test_upwind_selection_sign_convention():
    """c*Dx(u) on the cardinalised lhs takes the backward stencil for c > 0 (upwind_difference.jl:192-198)."""
    from molgpu.symbolic import Differential, Eq, Field, Interval, IV, Param, PDESystem, sin
    from molgpu.api import MOLFiniteDifference
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx = Differential(t), Differential(x)
    for c in (1.0, -1.0):
        cp = Param("c", c)
        s = PDESystem([Eq(Dt(u(x, t)), -cp * Dx(u(x, t)))],
                      [Eq(u(x, 0.0), sin(x)), Eq(u(0.0, t), u(1.0, t))],
                      [(t, Interval(0, 1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [cp])
        spec = s.to_spec(MOLFiniteDifference({x: 0.125}, t))
        orc = OracleProblem(spec)
        v = np.arange(orc.n_unknowns, dtype=float) ** 2
        du = orc.rhs(v, 0.0)
        n = orc.n_unknowns
        # interior point k (not wrapping): backward (v[k]-v[k-1]) for c>0, forward for c<0
        k = 3
        dx = 0.125
        expect = -c * ((v[k] - v[k - 1]) / dx if c > 0 else (v[k + 1] - v[k]) / dx)
        assert abs(du[k] - expect) < 1e-12 * abs(expect)
        di = DescInterp(lower(spec))
        assert np.allclose(di.rhs(v, 0.0), du, rtol=1e-15, atol=0)


def test_robin_and_dirichlet_time_dependent_rows():
    """a*u + b*Dx(u) = g(t) rows with time- and parameter-dependent data go through boundary programs."""
    from molgpu.symbolic import Differential, Eq, Field, Interval, IV, Param, PDESystem, sin
    from molgpu.api import MOLFiniteDifference
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    k = Param("k", 2.0)
    s = PDESystem([Eq(Dt(u(x, t)), Dxx(u(x, t)))],
                  [Eq(u(x, 0.0), sin(x)), Eq(2.0 * u(0.0, t) + 3.0 * Dx(u(0.0, t)), k * t),
                   Eq(u(1.0, t), t * t + 1.0)],
                  [(t, Interval(0, 1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [k])
    spec = s.to_spec(MOLFiniteDifference({x: 0.1}, t))
    lw = lower(spec)
    assert any(e["prog"] >= 0 for e in lw.bcs.values())
    orc = OracleProblem(spec)
    di = DescInterp(lw)
    v = np.random.default_rng(2).standard_normal(orc.n_unknowns)
    assert np.allclose(di.rhs(v, 0.7), orc.rhs(v, 0.7), rtol=1e-14, atol=1e-12)


def test_header_declares_every_exported_symbol():
    hdr = open(os.path.join(ROOT, "include", "molgpu.h")).read()
    declared = set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(mol_\w+)\(", hdr, re.M))
    assert declared == set(L.EXPORTED)


def test_library_loads_and_exports():
    """The C-ABI library loads without a GPU and exports every header symbol."""
    lib = L.lib()
    for name in L.EXPORTED:
        assert hasattr(lib, name)
    assert lib.mol_version() // 10000 == L.MOL_ABI_VERSION
    assert lib.mol_status_string(-6) == b"unsupported discretization"


def test_invalid_descriptor_rejected_before_device_work():
    """Malformed programs fail at plan creation with MOL_ERR_INVALID; validation touches no device."""
    from molgpu import Plan
    sys_, disc, _ = problems.heat1d(n=11)
    lw = lower(sys_.to_spec(disc))
    lw.programs[lw.cell_prog] = [(L.OP_CONST, 0, 0, 0, 0, 999)] + list(lw.programs[lw.cell_prog])
    with pytest.raises(L.MolError) as e:
        Plan(lw)
    assert e.value.status == -1 and "constant" in str(e.value)


def test_register_allocation_reuses_registers():
    """A long pointwise program fits in the 64-register file through reuse."""
    from molgpu.lowering import ProgramBuilder
    sys_, disc, _ = problems.heat1d(n=11)
    lw = lower(sys_.to_spec(disc))
    pb = ProgramBuilder(lw, "cell", L.MOL_MAX_REGS)
    tree = ("field", "u")
    for i in range(300):
        tree = ("add", ("mul", tree, ("num", 1.0 + i)), ("field", "u"))
    pb.out(tree, 0)
    code = pb.finish()
    assert max(max(r[1], r[2], r[3]) for r in code) < 8


@pytest.mark.parametrize("name,kw", [("brusselator", dict(N=8)), ("adr3d", dict(N=6, nz_pts=8))])
def test_generated_code_compiles_for_sm103a(name, kw):
    """generate_code + NVRTC compile of every kernel group, without a device."""
    from molgpu import Descriptor
    sys_, disc, _ = getattr(problems, name)(**kw)
    D = Descriptor(lower(sys_.to_spec(disc)))
    need = C.c_int64()
    assert L.lib().mol_generate_code(C.byref(D.desc), None, 0, C.byref(need)) == 0
    buf = C.create_string_buffer(need.value)
    assert L.lib().mol_generate_code(C.byref(D.desc), buf, need.value, C.byref(need)) == 0
    src = buf.value.decode()
    assert "gen_cell" in src
    # periodic dimensions use wrapped interior offsets, the others the interior fast path
    assert "wrap_line_ok" in src
    assert ("fast_nonlinlap" in src) == (name == "adr3d")  # z of the 3-D problem is Dirichlet
    log = C.create_string_buffer(1 << 16)
    st = L.lib().mol_codegen_compile_check(C.byref(D.desc), log, 1 << 16)
    assert st == 0, log.value.decode()


def _registered_bc_problem():
    """The boundary-condition docs' example: u(t, x, y_min) ~ f(t, x, y_min) + alpha / g(x, y_min)
    with f a plain function (traced) and g registered (a conditional on sin(x y) + cos(y))."""
    import math as _m
    from molgpu.api import MOLFiniteDifference
    from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, register
    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")

    def g_host(xx, yy):
        z = np.sin(xx * yy) + np.cos(yy)
        return np.where(z > 0, xx, 1.0)
    g = register("g_bc_doc", g_host)
    alpha = 9.0

    def f(tt, xx, yy):
        return xx * yy - tt
    Dt, Dxx, Dyy = Differential(t), Differential(x) ** 2, Differential(y) ** 2
    s = PDESystem([Eq(Dt(u(x, y, t)), Dxx(u(x, y, t)) + Dyy(u(x, y, t)))],
                  [Eq(u(x, y, 0.0), 1.0 + 0.1 * x * y), Eq(u(x, 0.0, t), f(t, x, 0.0) + alpha / g(x, 0.0)),
                   Eq(u(x, 1.0, t), 2.0), Eq(u(0.0, y, t), 1.0), Eq(u(1.0, y, t), 1.0 + t)],
                  [(t, Interval(0, 1)), (x, Interval(0.0, 1.0)), (y, Interval(0.0, 1.0))], [t, x, y], [u(x, y, t)])
    return s.to_spec(MOLFiniteDifference({x: 0.1, y: 0.125}, t))


def test_registered_function_in_a_boundary_row():
    spec = _registered_bc_problem()
    lw = lower(spec)
    orc = OracleProblem(spec)
    assert any(a.size == int(np.prod(lw.npts)) for a in lw.aux)    # host-evaluated on the face
    u = lw.u0 + 0.01 * np.random.default_rng(0).standard_normal(lw.n_unknowns)
    for t in (0.0, 0.6):
        a, b = orc.rhs(u, t), DescInterp(lw).rhs(u, t)
        assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a), t


def _third_derivative_problem(order):
    import math
    from molgpu.api import MOLFiniteDifference
    from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, sin
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx = Differential(t), Differential(x)
    s = PDESystem([Eq(Dt(u(x, t)), (Dx ** 2)(u(x, t)) + 0.3 * (Dx ** 3)(u(x, t)))],
                  [Eq(u(x, 0.0), sin(math.pi * x)), Eq(u(0.0, t), 0.0), Eq(Dx(u(1.0, t)), 0.0)],
                  [(t, Interval(0, 1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)])
    return s.to_spec(MOLFiniteDifference({x: 21}, t, approx_order=order))


@pytest.mark.parametrize("order", [3, 5, 7])
def test_odd_approx_order_warns_and_builds_its_tables(order):
    """An odd approx_order draws the reference's warning and is kept as given
    (MOLFiniteDifference.jl:56-58): the tables of that order, equal to the oracle's."""
    with pytest.warns(UserWarning, match="must be even"):
        spec = _third_derivative_problem(order)
    assert spec["disc"]["approx_order"] == order
    lw = lower(spec)
    orc = OracleProblem(spec)
    v = lw.u0 + 0.01 * np.random.default_rng(1).standard_normal(lw.n_unknowns)
    a, b = orc.rhs(v, 0.2), DescInterp(lw).rhs(v, 0.2)
    assert np.linalg.norm(a - b) <= 1e-14 * np.linalg.norm(a)


def test_approx_order_one_is_refused():
    """approx_order = 1 passes the constructor's bound (>= 1) with the odd-order warning, and
    the centered tables refuse it (centered_diff_weights.jl:8: approximation_order > 1)."""
    with pytest.warns(UserWarning):
        spec = _third_derivative_problem(1)
    with pytest.raises(ValueError, match="greater than 1"):
        lower(spec)
    from molgpu.api import MOLFiniteDifference
    with pytest.raises(ValueError):
        MOLFiniteDifference({"x": 11}, None, approx_order=0)
