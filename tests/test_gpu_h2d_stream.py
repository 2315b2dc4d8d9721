"""The first step of a call on a pinned host state streams the host-to-device copy in slabs
of the slowest dimension and runs stage 1 slab by slab behind it: the result equals stepping
a device copy of the state bit for bit (periodic, bounded and 3-D slowest dimensions, one
and several steps, generated code and interpreter)."""
import numpy as np
import pytest

from molgpu import Plan, lower, problems

pytestmark = pytest.mark.gpu

CASES = {
    "brusselator_periodic": lambda: problems.brusselator(N=256),
    "stretched_2d_bounded": lambda: problems.stretched_2d(nx=300, ny=260, order=4),
    "adr3d_dirichlet_z": lambda: problems.adr3d(N=48, nz_pts=50),
    "weno_bounded_x_periodic_y": lambda: problems.burgers_weno_channel(nx=300, ny=257),
}


@pytest.mark.parametrize("codegen", [True, False])
@pytest.mark.parametrize("nsteps", [1, 3])
@pytest.mark.parametrize("name", sorted(CASES))
def test_streamed_first_step_bit_identical(gpu_lib, monkeypatch, name, nsteps, codegen):
    torch = pytest.importorskip("torch")
    if not codegen:
        monkeypatch.setenv("MOL_DISABLE_CODEGEN", "1")
    monkeypatch.setenv("MOL_FACE_PASS", "0")
    s, d, ex = CASES[name]()
    lw = lower(s.to_spec(d))
    plan = Plan(lw)
    dt = ex.get("dt", ex.get("dt_ssprk", 1e-6))
    pinned = torch.empty(lw.n_unknowns, dtype=torch.float64, pin_memory=True)
    pinned.copy_(torch.from_numpy(lw.u0))
    h = pinned.numpy()
    plan.step_ssprk33(h, dt, nsteps, t0=0.2)
    dev = torch.tensor(lw.u0, device="cuda")
    torch.cuda.synchronize()
    plan.step_ssprk33(dev, dt, nsteps, t0=0.2)
    torch.cuda.synchronize()   # the plan's own stream does not order with torch's
    assert np.array_equal(h, dev.cpu().numpy()), name
    monkeypatch.setenv("MOL_H2D_SLABS", "0")
    pinned.copy_(torch.from_numpy(lw.u0))
    plan.step_ssprk33(h, dt, nsteps, t0=0.2)
    assert np.array_equal(h, dev.cpu().numpy()), name
    plan.close()


def test_streamed_first_step_f32state(gpu_lib, monkeypatch):
    """The Float32-state variant streams its copy the same way."""
    torch = pytest.importorskip("torch")
    s, d, ex = problems.brusselator(N=256)
    lw = lower(s.to_spec(d))
    plan = Plan(lw)
    dt = ex["dt_ssprk"]
    pinned = torch.empty(lw.n_unknowns, dtype=torch.float32, pin_memory=True)
    pinned.copy_(torch.from_numpy(lw.u0.astype(np.float32)))
    h = pinned.numpy()
    plan.step_ssprk33(h, dt, 2, t0=0.2)
    dev = torch.tensor(lw.u0.astype(np.float32), device="cuda")
    torch.cuda.synchronize()
    plan.step_ssprk33(dev, dt, 2, t0=0.2)
    torch.cuda.synchronize()
    assert np.array_equal(h, dev.cpu().numpy())
    plan.close()
