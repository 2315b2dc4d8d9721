"""Nonuniform grids on the GPU against the oracle: per-point centered rows (generated code and
interpreter), boundary rows built from the points, fixed SSPRK33 trajectories, Tsit5, the
discrete adjoint and the Float32-state variant (reference: centered_diff_weights.jl:77-153,
centered_difference.jl:32-56; the reference's test/Diffusion/MOL_1D_Linear_Diffusion.jl
Tests 00 and 03 build these operators)."""
import math

import numpy as np
import pytest

from molgpu import Plan, Tsit5, discretize, lower, problems, solve
from molgpu import _lib as L
from oracle.integrators import ssprk33, tsit5
from oracle.mol_oracle import OracleProblem

pytestmark = pytest.mark.gpu

CASES = {
    "stretched_o2": lambda: problems.stretched_reaction_diffusion(n=201, order=2),
    "stretched_o6": lambda: problems.stretched_reaction_diffusion(n=201, order=6),
    "neumann_cosine_o8": lambda: problems.neumann_cosine(n=300, order=8),
    "stretched_2d": lambda: problems.stretched_2d(nx=48, ny=40),
}


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _setup(name):
    s, d, ex = CASES[name]()
    spec = s.to_spec(d)
    return spec, lower(spec), OracleProblem(spec), ex


@pytest.mark.parametrize("name", sorted(CASES))
def test_nonuniform_rhs_and_trajectory(gpu_lib, name):
    spec, lw, orc, ex = _setup(name)
    plan = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(plan.handle) == 1
    v = lw.u0 + 0.05 * np.random.default_rng(4).standard_normal(lw.n_unknowns)
    for t in (0.0, 0.37):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, v, None, t)
        ref = orc.rhs(v, t)
        assert _rel(du, ref) <= 1e-12, (name, t)
    u = lw.u0.copy()
    plan.step_ssprk33(u, ex["dt"], 40, t0=0.1)
    ref, _ = ssprk33(lambda w, tt: orc.rhs(w, tt), lw.u0, 0.1, ex["dt"], 40)
    assert _rel(u, ref) <= 1e-10, name
    plan.close()


@pytest.mark.parametrize("name", ["stretched_o6", "stretched_2d"])
def test_nonuniform_generated_matches_interpreter(gpu_lib, name, monkeypatch):
    spec, lw, orc, ex = _setup(name)
    gen = Plan(lw)
    monkeypatch.setenv("MOL_DISABLE_CODEGEN", "1")
    interp = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(interp.handle) == 0
    u = lw.u0 * 1.01
    a, b = np.zeros_like(u), np.zeros_like(u)
    gen.rhs(a, u, None, 0.9)
    interp.rhs(b, u, None, 0.9)
    assert _rel(a, b) < 1e-13
    x, y = lw.u0.copy(), lw.u0.copy()
    gen.step_ssprk33(x, ex["dt"], 20)
    interp.step_ssprk33(y, ex["dt"], 20)
    assert _rel(x, y) < 1e-12


def test_nonuniform_tsit5_neumann_cosine(gpu_lib):
    """Order-8 Neumann problem solved adaptively: matches the oracle's Tsit5 and the exact
    solution exp(-t) cos x."""
    s, d, _ = problems.neumann_cosine(n=80, order=8)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    plan = Plan(lw)
    u = lw.u0.copy()
    st = plan.solve_tsit5(u, 0.0, 0.2, 1e-10, 1e-10)
    ref, rst = tsit5(lambda v, t: orc.rhs(v, t), lw.u0, 0.0, 0.2, 1e-10, 1e-10)
    assert _rel(u, ref) < 1e-9
    assert abs(st["naccept"] - rst["naccept"]) <= 2
    x = lw.grids[0][lw.lower[0]:lw.npts[0] - lw.upper[0]]
    assert np.max(np.abs(u - math.exp(-0.2) * np.cos(x))) < 1e-6
    plan.close()


def test_nonuniform_adjoint_matches_finite_differences(gpu_lib):
    spec, lw, orc, ex = _setup("stretched_o6")
    plan = Plan(lw)
    dt, n = ex["dt"], 30
    target = np.zeros(lw.n_unknowns)

    def loss(u0):
        u = u0.copy()
        plan.step_ssprk33(u, dt, n, t0=0.0)
        return 0.5 * float(np.sum((u - target) ** 2))

    g = np.zeros(lw.n_unknowns)
    plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=4, dLdu0=g)
    w = np.random.default_rng(9).standard_normal(lw.n_unknowns)
    h = 1e-6
    fd = (loss(lw.u0 + h * w) - loss(lw.u0 - h * w)) / (2 * h)
    assert abs(g @ w - fd) <= 1e-6 * abs(fd), (g @ w, fd)
    plan.close()


def test_nonuniform_f32state(gpu_lib):
    spec, lw, orc, ex = _setup("stretched_2d")
    plan = Plan(lw)
    u64 = lw.u0.copy()
    u32 = u64.astype(np.float32)
    plan.step_ssprk33(u64, ex["dt"], 20)
    plan.step_ssprk33(u32, ex["dt"], 20)
    assert _rel(u32.astype(np.float64), u64) < 1e-5
    plan.close()


@pytest.mark.parametrize("kind", ["symmetric", "left", "right", "chebyshev"])
def test_nonuniform_upwind_rhs_trajectory_and_boundedness(gpu_lib, kind):
    """First-order upwinding on the reference's clustered grids (stretching up to 1000): RHS
    and SSPRK33 trajectory against the oracle, and the reference test's boundedness over
    t in [0, 0.25] (test/Convection_NU/MOL_1D_Linear_Convection_NonUniform.jl)."""
    s, d, ex = problems.convection_nonuniform(kind, n=101)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    plan = Plan(lw)
    v = lw.u0 + 0.05 * np.random.default_rng(4).standard_normal(lw.n_unknowns)
    for t in (0.0, 0.11):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, v, None, t)
        ref = orc.rhs(v, t)
        assert _rel(du, ref) <= 1e-12, (kind, t)
    u = lw.u0.copy()
    plan.step_ssprk33(u, ex["dt"], 40, t0=0.0)
    ref, _ = ssprk33(lambda w, tt: orc.rhs(w, tt), lw.u0, 0.0, ex["dt"], 40)
    assert _rel(u, ref) <= 1e-10, kind
    nsteps = int(round(0.25 / ex["dt"]))
    u = lw.u0.copy()
    plan.step_ssprk33(u, ex["dt"], nsteps, t0=0.0)
    assert np.all(np.isfinite(u)) and np.max(np.abs(u)) < 5
    plan.close()


def test_nonuniform_upwind_adjoint_matches_finite_differences(gpu_lib):
    s, d, ex = problems.convection_nonuniform("chebyshev", n=101)
    lw = lower(s.to_spec(d))
    plan = Plan(lw)
    dt, n = ex["dt"], 30
    target = np.zeros(lw.n_unknowns)

    def loss(u0):
        u = u0.copy()
        plan.step_ssprk33(u, dt, n, t0=0.0)
        return 0.5 * float(np.sum((u - target) ** 2))

    g = np.zeros(lw.n_unknowns)
    plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=4, dLdu0=g)
    w = np.random.default_rng(9).standard_normal(lw.n_unknowns)
    h = 1e-6
    fd = (loss(lw.u0 + h * w) - loss(lw.u0 - h * w)) / (2 * h)
    assert abs(g @ w - fd) <= 1e-6 * abs(fd), (g @ w, fd)
    plan.close()


WENO_KINDS = ["uniform", "sinh", "tanh"]


@pytest.mark.parametrize("kind", WENO_KINDS)
def test_nonuniform_weno_rhs_and_trajectory(gpu_lib, kind):
    """Node-centred Lagrange WENO-5 on grids given as points (nonuniform_weno.jl): RHS and
    SSPRK33 trajectory against the oracle, generated code against the interpreter."""
    s, d, ex = problems.weno_convection_mms(kind, 161)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    plan = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(plan.handle) == 1
    v = lw.u0 + 0.05 * np.random.default_rng(4).standard_normal(lw.n_unknowns)
    for t in (0.0, 0.03):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, v, None, t)
        ref = orc.rhs(v, t)
        assert _rel(du, ref) <= 1e-12, (kind, t)
    u = lw.u0.copy()
    plan.step_ssprk33(u, ex["dt"], 40, t0=0.0)
    ref, _ = ssprk33(lambda w, tt: orc.rhs(w, tt), lw.u0, 0.0, ex["dt"], 40)
    assert _rel(u, ref) <= 1e-10, kind
    plan.close()


def test_nonuniform_weno_generated_matches_interpreter(gpu_lib, monkeypatch):
    s, d, ex = problems.weno_convection_mms("sinh", 161)
    lw = lower(s.to_spec(d))
    gen = Plan(lw)
    monkeypatch.setenv("MOL_DISABLE_CODEGEN", "1")
    interp = Plan(lw)
    u = lw.u0 * 1.01
    a, b = np.zeros_like(u), np.zeros_like(u)
    gen.rhs(a, u, None, 0.02)
    interp.rhs(b, u, None, 0.02)
    assert _rel(a, b) < 1e-13


def test_nonuniform_weno_solution_converges(gpu_lib):
    """The reference's MMS convergence run on the uniform points (CFL 0.01 to t = 0.05, SSPRK33;
    its assertion: observed order above 3.75)."""
    errs = []
    for n in (81, 161):
        s, d, ex = problems.weno_convection_mms("uniform", n)
        lw = lower(s.to_spec(d))
        plan = Plan(lw)
        nsteps = int(math.ceil(0.05 / ex["dt"]))
        dt = 0.05 / nsteps
        u = lw.u0.copy()
        plan.step_ssprk33(u, dt, nsteps, t0=0.0)
        xs = lw.grids[0]
        full = plan.fill_grid(u, 0.05)[0]
        w = np.concatenate([np.diff(xs), [xs[-1] - xs[-2]]])
        ue = problems.weno_mms_exact(xs, 0.05)
        errs.append(math.sqrt(np.sum(w * (full - ue) ** 2)) / math.sqrt(np.sum(w * ue ** 2)))
        plan.close()
    assert math.log(errs[0] / errs[1]) / math.log(160 / 80) > 3.75, errs


def test_nonuniform_weno_adjoint_matches_finite_differences(gpu_lib):
    s, d, ex = problems.weno_convection_mms("tanh", 81)
    lw = lower(s.to_spec(d))
    plan = Plan(lw)
    dt, n = ex["dt"] * 20, 25
    target = np.zeros(lw.n_unknowns)

    def loss(u0):
        u = u0.copy()
        plan.step_ssprk33(u, dt, n, t0=0.0)
        return 0.5 * float(np.sum((u - target) ** 2))

    g = np.zeros(lw.n_unknowns)
    plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=4, dLdu0=g)
    w = np.random.default_rng(9).standard_normal(lw.n_unknowns)

    def cd(h):
        return (loss(lw.u0 + h * w) - loss(lw.u0 - h * w)) / (2 * h)

    fd = (4.0 * cd(5e-7) - cd(1e-6)) / 3.0
    assert abs(g @ w - fd) <= 1e-6 * abs(fd), (g @ w, fd)
    plan.close()


def test_burgers_nonuniform_upwind_tsit5(gpu_lib):
    """The reference's nonuniform Burgers test (first-order upwinding on a perturbed grid,
    Tsit5 to t = 1; burgers_eq.jl:106-152 asserts atol 10^-2.5 against x/(t+1))."""
    s, d, _ = problems.burgers_nonuniform_upwind()
    prob = discretize(s, d)
    sol = solve(prob, Tsit5(), abstol=1e-8, reltol=1e-8, saveat=0.25)
    x = sol["x"]
    for i, t in enumerate(sol.ts):
        assert np.max(np.abs(sol["u"][i] - x / (t + 1))) < 10 ** -2.5, t


# the nonlinear Laplacian on a nonuniform grid (the reference's test/Nonlinear_Diffusion_NU):
# per-half-point tables, the outer operator on the grid's midpoints
NLD_CASES = [(2, "u2"), (4, "u2"), (2, "x"), (6, "x")]


@pytest.mark.parametrize("order,coefficient", NLD_CASES)
def test_nonuniform_nonlinlap_rhs_and_trajectory(gpu_lib, order, coefficient):
    s, d, ex = problems.nonlinear_diffusion_nonuniform(order, coefficient=coefficient)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    plan = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(plan.handle) == 1
    v = lw.u0 * (1 + 0.05 * np.random.default_rng(order).standard_normal(lw.n_unknowns))
    for t in (0.0, 0.7):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, v, None, t)
        assert _rel(du, orc.rhs(v, t)) < 1e-12, t
    u = lw.u0.copy()
    plan.step_ssprk33(u, ex["dt"], 40, t0=0.1)
    ref, _ = ssprk33(lambda w, tt: orc.rhs(w, tt), lw.u0, 0.1, ex["dt"], 40)
    assert _rel(u, ref) < 1e-10
    plan.close()


def test_nonuniform_nonlinlap_generated_matches_interpreter(gpu_lib, monkeypatch):
    """Generated code without and with the face pass (faces computed once per step by their
    own kernel) and the interpreter give the same right-hand side."""
    s, d, ex = problems.nonlinear_diffusion_nonuniform(4, coefficient="x")
    lw = lower(s.to_spec(d))
    gen = Plan(lw)
    monkeypatch.setenv("MOL_FACE_PASS", "1")
    faced = Plan(lw)
    monkeypatch.setenv("MOL_DISABLE_CODEGEN", "1")
    interp = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(interp.handle) == 0
    u = lw.u0 * 1.01
    a, b, c = np.zeros_like(u), np.zeros_like(u), np.zeros_like(u)
    gen.rhs(a, u, None, 0.9)
    faced.rhs(c, u, None, 0.9)
    interp.rhs(b, u, None, 0.9)
    assert _rel(a, b) < 1e-13 and _rel(c, b) < 1e-13
    x, y = lw.u0.copy(), lw.u0.copy()
    gen.step_ssprk33(x, ex["dt"], 20)
    faced.step_ssprk33(y, ex["dt"], 20)
    assert _rel(x, y) < 1e-13
    for pl in (gen, faced, interp):
        pl.close()


def test_nonuniform_nonlinlap_tracks_the_exact_solution(gpu_lib):
    """The reference's Test 01a (u_t = (u^2 u_x)_x, u = (x + 1/2)/(2 sqrt(50 - t)) on a jittered
    0:0.01:2) solved on the GPU with Tsit5 to t = 2: within 1e-6 of the exact solution (the
    reference test's bar is 0.1)."""
    s, d, ex = problems.nonlinear_diffusion_nonuniform(2)
    lw = lower(s.to_spec(d))
    plan = Plan(lw)
    u = lw.u0.copy()
    st = plan.solve_tsit5(u, 0.0, 2.0, 1e-8, 1e-8)
    assert st["t"] == 2.0
    exact = problems.nonlinear_diffusion_nu_exact(ex["points"][1:-1], 2.0)
    assert np.max(np.abs(u - exact)) < 1e-6
    plan.close()


def test_nonuniform_nonlinlap_adjoint_matches_finite_differences(gpu_lib):
    s, d, ex = problems.nonlinear_diffusion_nonuniform(2)
    lw = lower(s.to_spec(d))
    plan = Plan(lw)
    dt, n = ex["dt"], 20
    target = np.full(lw.n_unknowns, 0.1)

    def loss(u0):
        u = u0.copy()
        plan.step_ssprk33(u, dt, n, t0=0.0)
        return 0.5 * float(np.sum((u - target) ** 2))

    g = np.zeros(lw.n_unknowns)
    plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=4, dLdu0=g)
    w = np.random.default_rng(9).standard_normal(lw.n_unknowns)
    h = 1e-6
    fd = (loss(lw.u0 + h * w) - loss(lw.u0 - h * w)) / (2 * h)
    assert abs(g @ w - fd) <= 1e-6 * abs(fd), (g @ w, fd)
    plan.close()


@pytest.mark.parametrize("order", [2, 4])
def test_nonuniform_mixed_rhs_trajectory_and_adjoint(gpu_lib, order, monkeypatch):
    """Mixed derivatives on two nonuniform dimensions (per-point rows on both): RHS and SSPRK33
    trajectory against the oracle, generated code against the interpreter, and the discrete
    adjoint against central differences."""
    s, d, ex = problems.mixed_nonuniform(order=order)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    plan = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(plan.handle) == 1
    v = lw.u0 + 0.05 * np.random.default_rng(order).standard_normal(lw.n_unknowns)
    du = np.zeros(lw.n_unknowns)
    plan.rhs(du, v, None, 0.3)
    assert _rel(du, orc.rhs(v, 0.3)) < 1e-12
    u = lw.u0.copy()
    plan.step_ssprk33(u, ex["dt"], 30, t0=0.0)
    ref, _ = ssprk33(lambda w, tt: orc.rhs(w, tt), lw.u0, 0.0, ex["dt"], 30)
    assert _rel(u, ref) < 1e-10
    target = np.zeros(lw.n_unknowns)

    def loss(u0):
        w = u0.copy()
        plan.step_ssprk33(w, ex["dt"], 12, t0=0.0)
        return 0.5 * float(np.sum((w - target) ** 2))

    g = np.zeros(lw.n_unknowns)
    plan.adjoint_ssprk33(lw.u0, ex["dt"], 12, target, nsnap=3, dLdu0=g)
    w = np.random.default_rng(11).standard_normal(lw.n_unknowns)
    h = 1e-6
    fd = (loss(lw.u0 + h * w) - loss(lw.u0 - h * w)) / (2 * h)
    assert abs(g @ w - fd) <= 1e-6 * abs(fd), (g @ w, fd)
    monkeypatch.setenv("MOL_DISABLE_CODEGEN", "1")
    interp = Plan(lw)
    b = np.zeros(lw.n_unknowns)
    interp.rhs(b, v, None, 0.3)
    assert _rel(du, b) < 1e-13
    interp.close()
    plan.close()
