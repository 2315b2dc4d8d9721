"""Non-finite detection on the fixed-step paths (OrdinaryDiffEq's unstable_check: a NaN in
the state ends the solve with ReturnCode.Unstable).  The NaN is injected on the host into
the initial state or the parameters; nothing faults on the GPU: the last SSPRK33 stage ORs a
finite test of its outputs into a flag that the host reads."""
import numpy as np
import pytest

from molgpu import Batch, Plan, lower, problems
from molgpu import _lib as L

pytestmark = pytest.mark.gpu

NONFINITE = -3


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _bruss(N=48):
    sys_, disc, ex = problems.brusselator(N=N)
    return lower(sys_.to_spec(disc)), ex["dt_ssprk"]


def test_device_state_nan_reported_by_check(gpu_lib):
    torch = _torch()
    lw, dt = _bruss()
    plan = Plan(lw)
    u0 = lw.u0.copy()
    u0[777] = np.nan
    u = torch.tensor(u0, device="cuda")
    plan.step_ssprk33(u, dt, 3)           # asynchronous on device state: no error here
    with pytest.raises(L.MolError) as e:
        plan.check()
    assert e.value.status == NONFINITE
    plan.check()                          # the condition was cleared
    v = torch.tensor(lw.u0, device="cuda")
    plan.step_ssprk33(v, dt, 20)          # a finite run afterwards reports nothing
    plan.check()
    assert torch.isfinite(v).all()
    plan.close()


def test_host_state_nan_returns_nonfinite(gpu_lib):
    lw, dt = _bruss()
    plan = Plan(lw)
    u = lw.u0.copy()
    u[5] = np.inf
    with pytest.raises(L.MolError) as e:
        plan.step_ssprk33(u, dt, 2)
    assert e.value.status == NONFINITE
    w = lw.u0.copy()
    plan.step_ssprk33(w, dt, 2)           # clean state: no error, flag not sticky
    assert np.isfinite(w).all()
    plan.close()


def test_nan_parameter_detected(gpu_lib):
    torch = _torch()
    lw, dt = _bruss(64)                   # 8192 unknowns per field
    plan = Plan(lw)
    u = torch.tensor(lw.u0, device="cuda")
    p = torch.tensor([float("nan")], dtype=torch.float64, device="cuda")
    plan.step_ssprk33(u, dt, 1, p=p)
    with pytest.raises(L.MolError) as e:
        plan.check()
    assert e.value.status == NONFINITE
    plan.close()


def test_face_pass_plan_detects(gpu_lib):
    """A nonlinear-Laplacian plan large enough for the face pass (198^2 cells)."""
    torch = _torch()
    sys_, disc, _ = problems.nonlinear_diffusion(200, 1.0, 1000)
    lw = lower(sys_.to_spec(disc))
    dt = 0.125 / 199 ** 2 / float(np.max(lw.u0)) ** 2
    plan = Plan(lw)
    u0 = lw.u0.copy()
    u0[-1] = np.nan
    u = torch.tensor(u0, device="cuda")
    plan.step_ssprk33(u, dt, 2)
    with pytest.raises(L.MolError) as e:
        plan.check()
    assert e.value.status == NONFINITE
    plan.close()


@pytest.mark.parametrize("tile_cells", [512, -1])
def test_batch_member_nan_reported(gpu_lib, tile_cells):
    torch = _torch()
    lws, dts = [], []
    for (n, k, seed) in [(33, 0.5, 1000), (40, 1.0, 1001), (57, 1.5, 1002)]:
        sys_, disc, _ = problems.nonlinear_diffusion(n, k, seed)
        lw = lower(sys_.to_spec(disc))
        lws.append(lw)
        dts.append(0.125 / (n - 1) ** 2 / float(np.max(lw.u0)) ** 2)
    batch = Batch(lws)
    batch.tune(128, 2, tile_cells)
    parts = [lw.u0.copy() for lw in lws]
    parts[1][100] = np.nan
    u = torch.tensor(batch.pack(parts), device="cuda")
    batch.step_ssprk33(u, np.array(dts), 4)
    with pytest.raises(L.MolError) as e:
        batch.check()
    assert e.value.status == NONFINITE
    v = torch.tensor(batch.pack([lw.u0 for lw in lws]), device="cuda")
    batch.step_ssprk33(v, np.array(dts), 4)
    batch.check()                          # cleared, and a clean run reports nothing
    batch.close()


def test_adjoint_nan_initial_state(gpu_lib):
    torch = _torch()
    sys_, disc, ex = problems.burgers(npts=257)
    lw = lower(sys_.to_spec(disc))
    plan = Plan(lw)
    u0 = lw.u0.copy()
    u0[10] = np.nan
    g = torch.zeros(lw.n_unknowns, dtype=torch.float64, device="cuda")
    with pytest.raises(L.MolError) as e:
        plan.adjoint_ssprk33(torch.tensor(u0, device="cuda"), ex["dt"], 6, torch.tensor(ex["target"], device="cuda"),
                             nsnap=2, dLdu0=g)
    assert e.value.status == NONFINITE
    plan.close()
