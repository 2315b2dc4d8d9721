"""GPU parity: libmolgpu against the oracle, through the C ABI.

Bars: RHS within 1e-12 relative (norm-wise) of the reference's
discretisation; fixed-step SSPRK33 trajectories within 1e-10 relative.
"""
import math

import numpy as np
import pytest

from molgpu import Plan, lower, problems
from oracle.integrators import ssprk33, tsit5
from oracle.mol_oracle import OracleProblem

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
TRAJ_TOL = 1e-10


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _setup(name, **kw):
    sys_, disc, ex = getattr(problems, name)(**kw)
    spec = sys_.to_spec(disc)
    lw = lower(spec)
    return Plan(lw), OracleProblem(spec), lw, ex


CASES = [
    ("heat1d", dict(n=101)),
    ("heat1d", dict(n=7)),
    ("brusselator", dict(N=8)),
    ("brusselator", dict(N=64)),
    ("brusselator", dict(N=256)),
    ("burgers", dict(npts=65)),
    ("burgers", dict(npts=65537)),
    ("nonlinear_diffusion", dict(n=9, k=1.3, seed=1000)),
    ("nonlinear_diffusion", dict(n=33, k=0.4, seed=1001)),
    ("nonlinear_diffusion", dict(n=4, k=0.4, seed=1002)),
    ("adr3d", dict(N=8, nz_pts=10)),
    ("adr3d", dict(N=32, nz_pts=34)),
]


@pytest.mark.parametrize("name,kw", CASES)
def test_rhs_parity(gpu_lib, name, kw):
    plan, orc, lw, _ = _setup(name, **kw)
    rng = np.random.default_rng(11)
    u = lw.u0 * (1 + 0.05 * rng.standard_normal(lw.n_unknowns)) + 0.01 * rng.standard_normal(lw.n_unknowns)
    for t in (0.0, 1.7):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, u, None, t)
        ref = orc.rhs(u, t)
        assert _rel(du, ref) < RHS_TOL, (name, t, _rel(du, ref))


def test_rhs_parameters_runtime(gpu_lib):
    """p passed at call time (the ODEProblem's parameter vector) overrides the defaults."""
    plan, orc, lw, _ = _setup("brusselator", N=32)
    u = lw.u0.copy()
    p = np.array([3.5])
    du = np.zeros(lw.n_unknowns)
    plan.rhs(du, u, p, 0.2)
    assert _rel(du, orc.rhs(u, 0.2, p)) < RHS_TOL
    # the plan skips re-uploading unchanged host parameters: alternate values must all land
    for val in (3.5, 7.25, 7.25, 3.5, None):
        plan.rhs(du, u, None if val is None else np.array([val]), 0.2)
        ref = orc.rhs(u, 0.2, np.array([3.5 if val is None else val]))
        assert _rel(du, ref) < RHS_TOL, val


TRAJ = [
    ("brusselator", dict(N=32), 40, None),
    ("burgers", dict(npts=257), 60, None),
    ("nonlinear_diffusion", dict(n=17, k=1.1, seed=1003), 40, 1e-5),
    ("adr3d", dict(N=12, nz_pts=14), 20, None),
    ("heat1d", dict(n=21), 50, 1e-5),
]


@pytest.mark.parametrize("name,kw,nsteps,dt", TRAJ)
def test_ssprk33_trajectory(gpu_lib, name, kw, nsteps, dt):
    plan, orc, lw, ex = _setup(name, **kw)
    if dt is None:
        dt = ex.get("dt", ex.get("dt_ssprk", 1e-5))
    u = lw.u0.copy()
    plan.step_ssprk33(u, dt, nsteps, t0=1.0)
    ref, _ = ssprk33(lambda v, t: orc.rhs(v, t), lw.u0, 1.0, dt, nsteps)
    assert _rel(u, ref) < TRAJ_TOL, _rel(u, ref)


def test_ssprk33_graph_chunks_and_tail(gpu_lib):
    """Steps replayed as captured CUDA graphs (chunks of 16) plus a directly launched tail."""
    plan, orc, lw, ex = _setup("brusselator", N=16)
    dt = ex["dt_ssprk"]
    a = lw.u0.copy()
    plan.step_ssprk33(a, dt, 37, t0=1.05)
    b = lw.u0.copy()
    for k in range(37):
        plan.step_ssprk33(b, dt, 1, t0=1.05 + k * dt)
    ref, _ = ssprk33(lambda v, t: orc.rhs(v, t), lw.u0, 1.05, dt, 37)
    assert _rel(a, ref) < TRAJ_TOL
    assert _rel(a, b) < 1e-13


def test_tsit5_heat_exact(gpu_lib):
    """Config 1: u0 = sin(pi x) decays exactly as exp(lam t) in the semi-discrete system."""
    plan, orc, lw, _ = _setup("heat1d", n=101)
    u = lw.u0.copy()
    st = plan.solve_tsit5(u, 0.0, 0.1, 1e-10, 1e-10)
    dx = 0.01
    lam = -(4 / dx ** 2) * math.sin(math.pi * dx / 2) ** 2
    assert abs(st["t"] - 0.1) < 1e-15
    assert np.max(np.abs(u - math.exp(lam * 0.1) * lw.u0)) < 1e-9
    ref, rst = tsit5(lambda v, t: orc.rhs(v, t), lw.u0, 0.0, 0.1, 1e-10, 1e-10)
    assert _rel(u, ref) < 1e-9
    assert abs(st["naccept"] - rst["naccept"]) <= 2


def test_tsit5_brusselator_short(gpu_lib):
    plan, orc, lw, _ = _setup("brusselator", N=16)
    u = lw.u0.copy()
    st = plan.solve_tsit5(u, 0.0, 1.5, 1e-8, 1e-8)
    ref, rst = tsit5(lambda v, t: orc.rhs(v, t), lw.u0, 0.0, 1.5, 1e-8, 1e-8)
    assert _rel(u, ref) < 1e-7
    assert st["naccept"] > 10


def test_f32state_error_reported(gpu_lib):
    """Float32-state variant: same program in FP32; error against FP64 stays at FP32 level."""
    plan, orc, lw, ex = _setup("brusselator", N=64)
    u64 = lw.u0.copy()
    du64 = np.zeros_like(u64)
    plan.rhs(du64, u64, None, 0.3)
    u32 = u64.astype(np.float32)
    du32 = np.zeros_like(u32)
    plan.rhs(du32, u32, None, 0.3)
    assert _rel(du32.astype(np.float64), du64) < 1e-4
    dt = ex["dt_ssprk"]
    a = u64.copy()
    plan.step_ssprk33(a, dt, 20, t0=0.0)
    b = u32.copy()
    plan.step_ssprk33(b, dt, 20, t0=0.0)
    assert _rel(b.astype(np.float64), a) < 1e-5


def test_device_pointers_match_host(gpu_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    plan, orc, lw, ex = _setup("burgers", npts=1025)
    u = torch.tensor(lw.u0, device="cuda")
    du = torch.zeros_like(u)
    plan.rhs(du, u, None, 0.0)
    torch.cuda.synchronize()
    host = np.zeros(lw.n_unknowns)
    plan.rhs(host, lw.u0, None, 0.0)
    assert np.array_equal(du.cpu().numpy(), host)
    plan.step_ssprk33(u, ex["dt"], 33, t0=0.0)
    torch.cuda.synchronize()
    h = lw.u0.copy()
    plan.step_ssprk33(h, ex["dt"], 33, t0=0.0)
    assert np.array_equal(u.cpu().numpy(), h)


@pytest.mark.parametrize("name,kw", [("brusselator", dict(N=64)), ("burgers", dict(npts=1025)),
                                     ("nonlinear_diffusion", dict(n=33, k=0.7, seed=1004)),
                                     ("adr3d", dict(N=16, nz_pts=18))])
def test_generated_rhs_matches_interpreter(gpu_lib, name, kw, monkeypatch):
    """The generated straight-line RHS and the register-machine interpreter agree."""
    from molgpu import _lib as L
    sys_, disc, ex = getattr(problems, name)(**kw)
    lw = lower(sys_.to_spec(disc))
    gen = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(gen.handle) == 1, L.lib().mol_plan_codegen_source(gen.handle)
    monkeypatch.setenv("MOL_DISABLE_CODEGEN", "1")
    interp = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(interp.handle) == 0
    u = lw.u0 * 1.01
    a, b = np.zeros_like(u), np.zeros_like(u)
    gen.rhs(a, u, None, 0.9)
    interp.rhs(b, u, None, 0.9)
    assert _rel(a, b) < 1e-13
    dt = ex.get("dt", ex.get("dt_ssprk", 1e-6))
    x, y = lw.u0.copy(), lw.u0.copy()
    gen.step_ssprk33(x, dt, 20)
    interp.step_ssprk33(y, dt, 20)
    assert _rel(x, y) < 1e-12


@pytest.mark.parametrize("nsteps", [1, 2, 5, 40])
def test_pinned_host_state_zero_copy(gpu_lib, monkeypatch, nsteps):
    """The last stage writes a pinned host state's result straight over the host link (no
    bulk copy back); the result equals stepping a device array, and equals the copy path
    (MOL_ZERO_COPY=0), bit for bit."""
    torch = pytest.importorskip("torch")
    sys_, disc, ex = problems.brusselator(N=48)
    lw = lower(sys_.to_spec(disc))
    plan = Plan(lw)
    st = torch.cuda.Stream()
    plan.set_stream(st.cuda_stream)
    dt = ex["dt_ssprk"]
    dev = torch.tensor(lw.u0, device="cuda")
    plan.step_ssprk33(dev, dt, nsteps, t0=1.05)
    st.synchronize()
    ref = dev.cpu().numpy()
    for zc in ("1", "0"):
        monkeypatch.setenv("MOL_ZERO_COPY", zc)
        pinned = torch.empty(lw.n_unknowns, dtype=torch.float64, pin_memory=True)
        pinned.copy_(torch.from_numpy(lw.u0))
        hnp = pinned.numpy()
        plan.step_ssprk33(hnp, dt, nsteps, t0=1.05)
        assert np.array_equal(hnp, ref), (zc, nsteps)
    plan.close()


@pytest.mark.parametrize("name,kw", [("nonlinear_diffusion", dict(n=40, k=1.1, seed=1004)),
                                     ("adr3d", dict(N=12, nz_pts=14))])
def test_face_pass_matches_faces_in_cell(gpu_lib, monkeypatch, name, kw):
    """The face pass (each nonlinear-Laplacian face evaluated once per stage, the cells
    reading it) gives the same RHS and trajectory, bit for bit, as every cell evaluating
    its own faces."""
    sys_, disc, ex = getattr(problems, name)(**kw)
    lw = lower(sys_.to_spec(disc))
    dt = ex.get("dt") or 1e-7
    out = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("MOL_FACE_PASS", mode)
        plan = Plan(lw)
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, lw.u0, None, 0.3)
        u = lw.u0.copy()
        plan.step_ssprk33(u, dt, 20, t0=0.0)
        out[mode] = (du, u)
        plan.close()
    assert np.array_equal(out["1"][0], out["0"][0])
    assert np.array_equal(out["1"][1], out["0"][1])


def test_fp64_warp_rate_independent_of_active_lanes(gpu_lib):
    """The hardware fact the kernels are built around (mol_diag_fp64_rate): an FP64 warp
    instruction costs the same with 32 or 1 active lanes."""
    import ctypes as C
    from molgpu import _lib as L
    rates = {}
    for act in (32, 1):
        w, t = C.c_double(), C.c_double()
        assert L.lib().mol_diag_fp64_rate(act, C.byref(w), C.byref(t)) == 0
        assert w.value > 0 and t.value > 0
        rates[act] = w.value
    assert 0.8 < rates[1] / rates[32] < 1.25, rates


def test_readme_example_heat_equation(gpu_lib):
    """The README's example, end to end through the MethodOfLines-style API: discretize and
    solve with SSPRK33; the result decays like exp(-pi^2 t) sin(pi x)."""
    from molgpu import (Differential, Eq, Field, Interval, IV, MOLFiniteDifference, PDESystem, SSPRK33,
                        discretize, sin, solve)
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dxx = Differential(t), Differential(x) ** 2
    eq = Eq(Dt(u(x, t)), Dxx(u(x, t)))
    bcs = [Eq(u(x, 0.0), sin(math.pi * x)), Eq(u(0.0, t), 0.0), Eq(u(1.0, t), 0.0)]
    pdesys = PDESystem([eq], bcs, [(t, Interval(0.0, 0.1)), (x, Interval(0.0, 1.0))], [t, x], [u(x, t)], [])
    prob = discretize(pdesys, MOLFiniteDifference({x: 0.01}, t, approx_order=2))
    sol = solve(prob, SSPRK33(), dt=2e-5, saveat=0.02)
    xs = np.arange(1, 100) * 0.01
    exact = np.exp(-math.pi ** 2 * 0.1) * np.sin(math.pi * xs)
    assert np.max(np.abs(sol.u - exact)) < 1e-3 * np.max(np.abs(exact))
    assert sol[u].shape == (6, 101) and np.array_equal(sol[u][-1, 1:-1], sol.u)
    assert np.array_equal(sol[x], np.arange(101) * 0.01) or np.allclose(sol[x], np.arange(101) * 0.01, atol=1e-15)


def test_tsit5_small_problem_one_cta_matches_launch_per_stage(gpu_lib, monkeypatch):
    """Problems of at most 1024 unknowns run whole Tsit5 attempts in one CTA; the same solve
    through the launch-per-stage path takes the same steps (the error norm is summed in a
    different order, so accept/reject decisions may differ at the margin) to the same result."""
    plan, orc, lw, _ = _setup("heat1d", n=101)
    a = lw.u0.copy()
    sa = plan.solve_tsit5(a, 0.0, 0.1, 1e-10, 1e-10)
    monkeypatch.setenv("MOL_TSIT_NO_SMALL", "1")
    b = lw.u0.copy()
    sb = plan.solve_tsit5(b, 0.0, 0.1, 1e-10, 1e-10)
    assert abs(sa["naccept"] - sb["naccept"]) <= 2 and abs(sa["t"] - 0.1) < 1e-15
    assert _rel(a, b) < 1e-12
    plan.close()
