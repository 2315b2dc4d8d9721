"""Coefficient stencils: a diffusion term with a coordinate-dependent coefficient,
Dj(K(x) Dj u), and the constant-coefficient first-derivative terms beside it (the 3-D ADR
system: nonlinear Laplacians with face diffusivities, the mixed term, upwinding) evaluated
from per-cell weights filled once at plan creation, in the difference form (default) and the
expanded form (MOL_FLAG_EXPAND_STENCILS).

Both forms against the numpy oracle at the parity bars (RHS 1e-12, fixed-step trajectories
1e-10, relative, norm-wise); the face pass is no longer launched for such problems.
"""
import numpy as np
import pytest

from molgpu import Plan, lower, problems
from molgpu import _lib as L
from oracle.integrators import ssprk33
from oracle.mol_oracle import OracleProblem

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
TRAJ_TOL = 1e-10


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _adr(N):
    sys_, disc, ex = problems.adr3d(N=N, nz_pts=N + 2)
    spec = sys_.to_spec(disc)
    return lower(spec), OracleProblem(spec), ex


@pytest.mark.parametrize("expand", [False, True])
@pytest.mark.parametrize("N", [8, 32])
def test_adr_rhs_both_forms(gpu_lib, N, expand):
    lw, orc, _ = _adr(N)
    plan = Plan(lw, expand_stencils=expand)
    rng = np.random.default_rng(21)
    u = lw.u0 * (1 + 0.05 * rng.standard_normal(lw.n_unknowns)) + 0.01 * rng.standard_normal(lw.n_unknowns)
    du = np.zeros(lw.n_unknowns)
    plan.rhs(du, u, None, 0.3)
    assert _rel(du, orc.rhs(u, 0.3)) < RHS_TOL
    plan.close()


@pytest.mark.parametrize("expand", [False, True])
def test_adr_trajectory_both_forms(gpu_lib, expand):
    lw, orc, ex = _adr(12)
    plan = Plan(lw, expand_stencils=expand)
    u = lw.u0.copy()
    plan.step_ssprk33(u, ex["dt"], 20, t0=0.0)
    ref, _ = ssprk33(lambda v, t: orc.rhs(v, t), lw.u0, 0.0, ex["dt"], 20)
    assert _rel(u, ref) < TRAJ_TOL
    plan.close()


def test_adr_forms_agree_with_each_other(gpu_lib):
    """Difference form and expanded form on the same state: two evaluations of one
    discretisation agree with each other and with the oracle to the RHS bar."""
    lw, orc, _ = _adr(32)
    rng = np.random.default_rng(22)
    u = lw.u0 + 0.01 * rng.standard_normal(lw.n_unknowns)
    out = []
    for expand in (False, True):
        plan = Plan(lw, expand_stencils=expand)
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, u, None, 0.0)
        out.append(du)
        plan.close()
    assert _rel(out[0], out[1]) < RHS_TOL
    ref = orc.rhs(u, 0.0)
    assert _rel(out[0], ref) < RHS_TOL and _rel(out[1], ref) < RHS_TOL


def test_adr_rhs_launches_no_face_pass(gpu_lib):
    """At 32^3 cells (where the face pass would start) the RHS is one launch: every
    nonlinear Laplacian of the ADR system is inside the coefficient stencil."""
    torch = _torch()
    lw, orc, _ = _adr(32)
    plan = Plan(lw)
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    u = torch.tensor(lw.u0, device="cuda")
    dd = torch.zeros_like(u)
    before = L.lib().mol_launch_count()
    plan.rhs(dd, u, None, 0.0)
    torch.cuda.synchronize()
    assert L.lib().mol_launch_count() - before == 1
    assert _rel(dd.cpu().numpy(), orc.rhs(lw.u0, 0.0)) < RHS_TOL
    plan.close()


def test_nonlinear_diffusion_keeps_face_pass(gpu_lib):
    """A coefficient that depends on the state (u^2) is not a coefficient stencil: the face
    pass still runs (two launches per RHS at 200^2 cells) and parity holds."""
    sys_, disc, _ = problems.nonlinear_diffusion(202, 1.3, 1000)
    spec = sys_.to_spec(disc)
    lw = lower(spec)
    torch = _torch()
    plan = Plan(lw)
    plan.set_stream(torch.cuda.current_stream().cuda_stream)
    u = torch.tensor(lw.u0, device="cuda")
    dd = torch.zeros_like(u)
    plan.rhs(dd, u, None, 0.0)
    torch.cuda.synchronize()
    before = L.lib().mol_launch_count()
    plan.rhs(dd, u, None, 0.0)
    torch.cuda.synchronize()
    assert L.lib().mol_launch_count() - before == 2
    assert _rel(dd.cpu().numpy(), OracleProblem(spec).rhs(lw.u0, 0.0)) < RHS_TOL
    plan.close()


@pytest.mark.parametrize("expand", [False, True])
def test_adr_vjp_both_forms_against_finite_differences(gpu_lib, expand):
    """The coefficient stencil's own VJP (per-tap scatter of the seed times the cell's weights,
    and the derivative with respect to each face's K) against central differences of the RHS
    along seeded directions, in u and in the face-diffusivity arrays."""
    import copy
    lw, _, _ = _adr(12)
    plan = Plan(lw, expand_stencils=expand)
    assert plan.coef_arrays == (7 if expand else 6)
    rng = np.random.default_rng(23)
    u = lw.u0 + 0.05 * rng.standard_normal(lw.n_unknowns)
    lam = rng.standard_normal(lw.n_unknowns)
    v = rng.standard_normal(lw.n_unknowns)
    lam_u = np.zeros(lw.n_unknowns)
    lam_aux = np.zeros(sum(a.size for a in lw.aux))
    plan.vjp(lam, u, None, 0.1, lam_u=lam_u, lam_aux=lam_aux)

    def rhs(pl, x):
        du = np.zeros_like(x)
        pl.rhs(du, x, None, 0.1)
        return du

    h = 1e-6
    fd = lam @ (rhs(plan, u + h * v) - rhs(plan, u - h * v)) / (2 * h)
    assert abs(lam_u @ v - fd) <= 1e-6 * abs(fd), (lam_u @ v, fd)
    dirs = [rng.standard_normal(a.size) * (a != 0) for a in lw.aux]
    ha = 1e-7

    def with_aux(sign):
        lw2 = copy.copy(lw)
        lw2.aux = [a + sign * ha * d for a, d in zip(lw.aux, dirs)]
        p2 = Plan(lw2, expand_stencils=expand)
        out = rhs(p2, u)
        p2.close()
        return out

    fda = lam @ (with_aux(+1) - with_aux(-1)) / (2 * ha)
    got = lam_aux @ np.concatenate(dirs)
    assert abs(got - fda) <= 1e-6 * abs(fda), (got, fda)
    plan.close()


@pytest.mark.parametrize("expand", [False, True])
def test_adr_adjoint_dLdK_both_forms(gpu_lib, expand):
    """dL/dK of a 6-step SSPRK33 misfit through the checkpointed adjoint, against a central
    difference of the loss along a seeded direction of the face arrays."""
    import copy
    lw, _, ex = _adr(12)
    rng = np.random.default_rng(24)
    target = rng.standard_normal(lw.n_unknowns) * 1e-3
    dt, n = ex["dt"], 6
    plan = Plan(lw, expand_stencils=expand)
    gaux = np.zeros(sum(a.size for a in lw.aux))
    loss, _ = plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=2, dLdaux=gaux)
    plan.close()
    dirs = [rng.standard_normal(a.size) * (a != 0) for a in lw.aux]
    h = 1e-7

    def L(sign):
        lw2 = copy.copy(lw)
        lw2.aux = [a + sign * h * d for a, d in zip(lw.aux, dirs)]
        p2 = Plan(lw2, expand_stencils=expand)
        w = lw.u0.copy()
        p2.step_ssprk33(w, dt, n)
        p2.close()
        return 0.5 * float(np.sum((w - target) ** 2))

    fd = (L(+1) - L(-1)) / (2 * h)
    got = gaux @ np.concatenate(dirs)
    assert abs(got - fd) <= 1e-6 * abs(fd), (got, fd)


@pytest.mark.parametrize("expand", [False, True])
def test_adr_f32state_reads_float_coefficients(gpu_lib, expand):
    """The Float32-state kernels read the FP32 copy of the coefficient arrays: their RHS and
    20 SSPRK33 steps stay at FP32 distance from the FP64 ones."""
    lw, _, ex = _adr(32)
    plan = Plan(lw, expand_stencils=expand)
    u64 = lw.u0.copy()
    du64 = np.zeros_like(u64)
    plan.rhs(du64, u64, None, 0.0)
    u32 = u64.astype(np.float32)
    du32 = np.zeros_like(u32)
    plan.rhs(du32, u32, None, 0.0)
    assert _rel(du32.astype(np.float64), du64) < 1e-4
    a = u64.copy()
    plan.step_ssprk33(a, ex["dt"], 20)
    b = u32.copy()
    plan.step_ssprk33(b, ex["dt"], 20)
    assert _rel(b.astype(np.float64), a) < 1e-5
    plan.close()


def _system(n):
    sys_, disc, ex = problems.coefficient_system(n)
    spec = sys_.to_spec(disc)
    return lower(spec), OracleProblem(spec), ex


@pytest.mark.parametrize("expand", [False, True])
def test_two_field_system_rhs_and_trajectory(gpu_lib, expand):
    """Two fields, each with its own coefficient stencil (arrays at different offsets), a
    parameter-scaled diffusivity left on the face form beside them, and Dirichlet, Neumann and
    Robin rows on every side (edge cells on the original statements)."""
    lw, orc, ex = _system(24)
    plan = Plan(lw, expand_stencils=expand)
    assert plan.coef_arrays == (2 + 4 if not expand else 3 + 5)
    rng = np.random.default_rng(25)
    u = lw.u0 * (1 + 0.05 * rng.standard_normal(lw.n_unknowns))
    for t in (0.0, 0.4):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, u, None, t)
        assert _rel(du, orc.rhs(u, t)) < RHS_TOL
    w = lw.u0.copy()
    plan.step_ssprk33(w, ex["dt"], 20, t0=0.0)
    ref, _ = ssprk33(lambda q, t: orc.rhs(q, t), lw.u0, 0.0, ex["dt"], 20)
    assert _rel(w, ref) < TRAJ_TOL
    plan.close()


@pytest.mark.parametrize("expand", [False, True])
def test_two_field_system_vjp(gpu_lib, expand):
    import copy
    lw, _, _ = _system(24)
    plan = Plan(lw, expand_stencils=expand)
    rng = np.random.default_rng(26)
    u = lw.u0 * (1 + 0.05 * rng.standard_normal(lw.n_unknowns))
    lam = rng.standard_normal(lw.n_unknowns)
    v = rng.standard_normal(lw.n_unknowns)
    lam_u = np.zeros(lw.n_unknowns)
    lam_p = np.zeros(1)
    lam_aux = np.zeros(sum(a.size for a in lw.aux))
    plan.vjp(lam, u, None, 0.2, lam_u=lam_u, lam_p=lam_p, lam_aux=lam_aux)

    def rhs(pl, x, p=None):
        du = np.zeros_like(x)
        pl.rhs(du, x, p, 0.2)
        return du

    h = 1e-6
    fd = lam @ (rhs(plan, u + h * v) - rhs(plan, u - h * v)) / (2 * h)
    assert abs(lam_u @ v - fd) <= 1e-6 * abs(fd), (lam_u @ v, fd)
    p0 = lw.param_values.copy()
    fdp = lam @ (rhs(plan, u, p0 + h) - rhs(plan, u, p0 - h)) / (2 * h)
    assert abs(lam_p[0] - fdp) <= 1e-6 * abs(fdp), (lam_p[0], fdp)
    dirs = [rng.standard_normal(a.size) * (a != 0) for a in lw.aux]

    def with_aux(sign):
        lw2 = copy.copy(lw)
        lw2.aux = [a + sign * 1e-7 * d for a, d in zip(lw.aux, dirs)]
        p2 = Plan(lw2, expand_stencils=expand)
        out = rhs(p2, u)
        p2.close()
        return out

    fda = lam @ (with_aux(+1) - with_aux(-1)) / 2e-7
    got = lam_aux @ np.concatenate(dirs)
    assert abs(got - fda) <= 1e-6 * abs(fda), (got, fda)
    plan.close()


def test_two_field_system_with_face_pass(gpu_lib):
    """At 200^2 cells per field the parameter-scaled term goes through the face pass while the
    other three diffusion terms are coefficient stencils; RHS against the oracle."""
    lw, orc, _ = _system(202)
    plan = Plan(lw)
    rng = np.random.default_rng(27)
    u = lw.u0 * (1 + 0.05 * rng.standard_normal(lw.n_unknowns))
    du = np.zeros(lw.n_unknowns)
    plan.rhs(du, u, None, 0.1)
    assert _rel(du, orc.rhs(u, 0.1)) < RHS_TOL
    plan.close()
