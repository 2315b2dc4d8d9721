"""Parity at the configurations' own sizes: the paths only large grids take (the streamed
host-to-device copy in slabs, the face pass, the ensemble's tile table over all 4096 members,
long binomial-checkpoint schedules) checked where the benchmark numbers are quoted.

References: the oracle's C/OpenMP restatements (oracle/c, themselves checked against the
numpy oracle in tests/test_oracle_c.py) where the numpy oracle would take minutes, the numpy
oracle elsewhere, central finite differences for gradients.  Bars as in test_gpu_parity:
RHS 1e-12, fixed-step trajectories 1e-10, gradients 1e-6 (all relative, norm-wise).
"""
import numpy as np
import pytest

from molgpu import Batch, Plan, lower, problems
from oracle.c_port import ADR3D, Brusselator
from oracle.integrators import ssprk33
from oracle.mol_oracle import OracleProblem

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-12
TRAJ_TOL = 1e-10
GRAD_TOL = 1e-6


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _on_stream(obj, torch):
    """Run a plan or batch on torch's current stream, so its asynchronous work on device
    tensors is ordered with the torch operations that produce and read them."""
    obj.set_stream(torch.cuda.current_stream().cuda_stream)
    return obj


@pytest.fixture(scope="module")
def bruss1024():
    sys_, disc, ex = problems.brusselator(N=1024)
    lw = lower(sys_.to_spec(disc))
    return lw, ex["dt_ssprk"], Brusselator(lw)


@pytest.fixture(scope="module")
def adr256():
    sys_, disc, ex = problems.adr3d(N=256, nz_pts=258)
    lw = lower(sys_.to_spec(disc))
    return lw, ex["dt"], ADR3D(lw)


def test_brusselator_1024_rhs_and_steps(gpu_lib, bruss1024):
    torch = _torch()
    lw, dt, cref = bruss1024
    plan = _on_stream(Plan(lw), torch)
    u = torch.tensor(lw.u0, device="cuda")
    du = torch.zeros_like(u)
    for t in (0.5, 1.2):                       # before and after the forcing switches on
        plan.rhs(du, u, None, t)
        assert _rel(du.cpu().numpy(), cref.rhs(lw.u0, t)) < RHS_TOL
    plan.step_ssprk33(u, dt, 20, t0=1.0)       # one 16-step graph chunk and 4 direct steps
    ref = cref.ssprk33(lw.u0, 1.0, dt, 20)
    assert _rel(u.cpu().numpy(), ref) < TRAJ_TOL
    plan.close()


def test_brusselator_1024_pinned_host_state(gpu_lib, bruss1024):
    """Pinned host state: the copy in streamed in slabs behind stage 1, the last stage writing
    the result straight back into host memory, call after call."""
    torch = _torch()
    lw, dt, cref = bruss1024
    plan = Plan(lw)
    host = torch.empty(lw.n_unknowns, dtype=torch.float64, pin_memory=True)
    host.copy_(torch.from_numpy(lw.u0))
    hnp = host.numpy()
    t = 1.0
    for n in (1, 1, 5):
        plan.step_ssprk33(hnp, dt, n, t0=t)
        t += n * dt
    ref = cref.ssprk33(lw.u0, 1.0, dt, 7)
    assert _rel(hnp, ref) < TRAJ_TOL
    plan.close()


@pytest.mark.parametrize("expand", [False, True])
def test_adr3d_256_rhs_and_steps(gpu_lib, adr256, expand):
    """The headline workload: RHS through the coefficient stencils (difference and expanded
    forms), SSPRK33 steps, device state."""
    torch = _torch()
    lw, dt, cref = adr256
    plan = _on_stream(Plan(lw, expand_stencils=expand), torch)
    u = torch.tensor(lw.u0, device="cuda")
    du = torch.zeros_like(u)
    plan.rhs(du, u, None, 0.1)
    assert _rel(du.cpu().numpy(), cref.rhs(lw.u0)) < RHS_TOL
    plan.step_ssprk33(u, dt, 5)
    ref = cref.ssprk33(lw.u0, dt, 5)
    assert _rel(u.cpu().numpy(), ref) < TRAJ_TOL
    plan.close()


@pytest.mark.parametrize("expand", [False, True])
def test_adr3d_256_pinned_host_state(gpu_lib, adr256, expand):
    torch = _torch()
    lw, dt, cref = adr256
    plan = Plan(lw, expand_stencils=expand)
    host = torch.empty(lw.n_unknowns, dtype=torch.float64, pin_memory=True)
    host.copy_(torch.from_numpy(lw.u0))
    hnp = host.numpy()
    plan.step_ssprk33(hnp, dt, 1)
    plan.step_ssprk33(hnp, dt, 2, t0=dt)
    ref = cref.ssprk33(lw.u0, dt, 3)
    assert _rel(hnp, ref) < TRAJ_TOL
    plan.close()


@pytest.mark.parametrize("expand", [False, True])
def test_adr3d_128_rhs_against_numpy_oracle(gpu_lib, expand):
    sys_, disc, _ = problems.adr3d(N=128, nz_pts=130)
    spec = sys_.to_spec(disc)
    lw = lower(spec)
    plan = Plan(lw, expand_stencils=expand)
    rng = np.random.default_rng(3)
    u = lw.u0 + 0.01 * rng.standard_normal(lw.n_unknowns)
    du = np.zeros(lw.n_unknowns)
    plan.rhs(du, u, None, 0.0)
    assert _rel(du, OracleProblem(spec).rhs(u, 0.0)) < RHS_TOL
    plan.close()


def test_ensemble_4096_members(gpu_lib):
    """One full launch of the configuration's 4096 uneven members (3 steps), 32 members spread
    over the size range against their own numpy-oracle trajectories."""
    torch = _torch()
    members = problems.ensemble_members(4096)
    lws, dts, specs = [], [], []
    for (n, k, seed) in members:
        sys_, disc, _ = problems.nonlinear_diffusion(n, k, seed)
        spec = sys_.to_spec(disc)
        lw = lower(spec)
        lws.append(lw)
        specs.append(spec)
        dts.append(0.125 / (n - 1) ** 2 / float(np.max(lw.u0)) ** 2)
    dts = np.array(dts)
    batch = _on_stream(Batch(lws), torch)
    u = torch.tensor(batch.pack([lw.u0 for lw in lws]), device="cuda")
    batch.step_ssprk33(u, dts, 3)
    batch.check()
    got = u.cpu().numpy()
    sizes = np.array([m[0] for m in members])
    order = np.argsort(sizes, kind="stable")
    picks = sorted(set(int(order[q]) for q in np.linspace(0, len(order) - 1, 32).round().astype(int)))
    assert sizes[picks].min() <= 33 and sizes[picks].max() >= 500
    for i in picks:
        orc = OracleProblem(specs[i])
        ref, _ = ssprk33(lambda v, t: orc.rhs(v, t), lws[i].u0, 0.0, dts[i], 3)
        assert _rel(got[batch.offsets[i]:batch.offsets[i + 1]], ref) < TRAJ_TOL, (i, members[i])
    batch.close()


def test_burgers_65536_gradient_64_snapshots(gpu_lib):
    """dL/du0 and dL/dnu of 200 steps with the configuration's 64 binomial snapshots, against
    central differences of the loss along a seeded direction (and in nu)."""
    torch = _torch()
    sys_, disc, ex = problems.burgers()
    lw = lower(sys_.to_spec(disc))
    plan = _on_stream(Plan(lw), torch)
    n, dt, steps = lw.n_unknowns, ex["dt"], 200
    tgt = torch.tensor(ex["target"], device="cuda")
    u0 = torch.tensor(lw.u0, device="cuda")
    g = torch.zeros(n, dtype=torch.float64, device="cuda")
    gp = torch.zeros(1, dtype=torch.float64, device="cuda")
    loss, nfw = plan.adjoint_ssprk33(u0, dt, steps, tgt, nsnap=64, dLdu0=g, dLdp=gp)
    assert nfw > steps                             # the schedule recomputed forward steps

    def L(u_start, nu):
        w = u_start.clone()
        plan.step_ssprk33(w, dt, steps, p=torch.tensor([nu], dtype=torch.float64, device="cuda"))
        return 0.5 * float(torch.sum((w - tgt) ** 2))

    nu = float(lw.param_values[0])
    assert abs(L(u0, nu) - loss) <= 1e-12 * abs(loss)
    v = torch.tensor(np.random.default_rng(5).standard_normal(n), device="cuda")
    eps = 1e-6 * max(1.0, float(torch.max(torch.abs(u0))))
    fd = (L(u0 + eps * v, nu) - L(u0 - eps * v, nu)) / (2 * eps)
    ad = float(torch.dot(g, v))
    assert abs(fd - ad) <= GRAD_TOL * abs(ad), (fd, ad)
    h = 1e-6 * max(1.0, nu)
    fdn = (L(u0, nu + h) - L(u0, nu - h)) / (2 * h)
    assert abs(fdn - float(gp.item())) <= GRAD_TOL * abs(float(gp.item())), (fdn, float(gp.item()))
    plan.close()
