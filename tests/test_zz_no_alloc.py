"""The allocation-free SSPRK33 entry point (mol_step_ssprk33_noalloc).

Callers that cannot let a call allocate device memory (a device-memory budget
fixed up front, host callbacks where CUDA allocation calls are not allowed) use
it instead of mol_step_ssprk33.  This file
is collected last so a run that stops at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from molgpu import Plan, lower, problems
from molgpu import _lib as L

pytestmark = pytest.mark.gpu

TOL = 1e-13  # same arithmetic as mol_step_ssprk33; only the stage buffers move


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


@pytest.mark.parametrize("name,kw", [("brusselator", dict(N=64)), ("burgers", dict(npts=4097))])
def test_noalloc_matches_step_ssprk33_two_calls(gpu_lib, name, kw):
    torch = _torch()
    sys_, disc, ex = getattr(problems, name)(**kw)
    lw = lower(sys_.to_spec(disc))
    dt = ex.get("dt", ex.get("dt_ssprk"))
    a = Plan(lw)
    b = Plan(lw)
    ua = torch.tensor(lw.u0, device="cuda")
    ub = torch.tensor(lw.u0, device="cuda")
    p = torch.tensor(lw.param_values, device="cuda")
    # two calls in a row on each path, the second continuing from the first
    a.step_ssprk33_noalloc(ua, dt, 7, t0=0.0, p=p)
    b.step_ssprk33(ub, dt, 7, t0=0.0, p=p)
    torch.cuda.synchronize()
    x, y = ua.cpu().numpy(), ub.cpu().numpy()
    assert np.linalg.norm(x - y) <= TOL * np.linalg.norm(y)
    a.step_ssprk33_noalloc(ua, dt, 5, t0=7 * dt, p=p)
    b.step_ssprk33(ub, dt, 5, t0=7 * dt, p=p)
    torch.cuda.synchronize()
    x, y = ua.cpu().numpy(), ub.cpu().numpy()
    assert np.linalg.norm(x - y) <= TOL * np.linalg.norm(y)
    a.close()
    b.close()


@pytest.mark.parametrize("face_buffer_first", [False, True])
def test_noalloc_nonlinear_laplacian(gpu_lib, face_buffer_first):
    """A nonlinear-Laplacian plan above the face-pass size (198 x 198 cells): on a fresh plan
    the allocation-free steps evaluate every face in the cell; after an ordinary step has
    made the plan's face buffer they read it.  Both must match mol_step_ssprk33."""
    torch = _torch()
    sys_, disc, _ = problems.nonlinear_diffusion(200, 1.3, 1000)
    lw = lower(sys_.to_spec(disc))
    dx = 1.0 / 199
    dt = 0.125 * dx * dx / float(np.max(lw.u0)) ** 2
    a = Plan(lw)
    b = Plan(lw)
    p = torch.tensor(lw.param_values, device="cuda")
    if face_buffer_first:
        w = torch.tensor(lw.u0, device="cuda")
        a.step_ssprk33(w, dt, 1, t0=0.0, p=p)       # makes plan a's face buffer
    ua = torch.tensor(lw.u0, device="cuda")
    ub = torch.tensor(lw.u0, device="cuda")
    for t0, n in ((0.0, 6), (6 * dt, 4)):
        a.step_ssprk33_noalloc(ua, dt, n, t0=t0, p=p)
        b.step_ssprk33(ub, dt, n, t0=t0, p=p)
        torch.cuda.synchronize()
        x, y = ua.cpu().numpy(), ub.cpu().numpy()
        assert np.linalg.norm(x - y) <= TOL * np.linalg.norm(y)
    a.close()
    b.close()


def test_noalloc_allocates_nothing_and_replays_from_a_cuda_graph(gpu_lib):
    """After one warm-up call (the scratch address lookup) the allocation-free steps leave the
    device's free memory unchanged, and they capture into a CUDA graph on the plan's stream:
    two replays (each restarting at t0) give what two mol_step_ssprk33 calls give."""
    torch = _torch()
    sys_, disc, ex = problems.brusselator(N=64)
    lw = lower(sys_.to_spec(disc))
    dt = ex["dt_ssprk"]
    s = torch.cuda.Stream()
    a = Plan(lw)
    a.set_stream(s.cuda_stream)
    b = Plan(lw)
    ua = torch.tensor(lw.u0, device="cuda")
    ub = torch.tensor(lw.u0, device="cuda")
    u0 = torch.tensor(lw.u0, device="cuda")
    a.step_ssprk33_noalloc(ua, dt, 1)                     # warm-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    a.step_ssprk33_noalloc(ua, dt, 3, t0=dt)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    ua.copy_(u0)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
        a.step_ssprk33_noalloc(ua, dt, 4, t0=0.0)
    for _ in range(2):
        g.replay()
        b.step_ssprk33(ub, dt, 4, t0=0.0)
    torch.cuda.synchronize()
    x, y = ua.cpu().numpy(), ub.cpu().numpy()
    assert np.linalg.norm(x - y) <= TOL * np.linalg.norm(y)
    assert np.linalg.norm(x - lw.u0) > 0
    del g
    a.close()
    b.close()


def test_noalloc_rejects_oversized_and_host_arrays(gpu_lib):
    torch = _torch()
    sys_, disc, ex = problems.brusselator(N=1024)       # 2,097,152 unknowns > 2^20
    big = Plan(lower(sys_.to_spec(disc)))
    u = torch.zeros(big.n, dtype=torch.float64, device="cuda")
    with pytest.raises(L.MolError) as e:
        big.step_ssprk33_noalloc(u, 1e-9, 1)
    assert e.value.status == -1 and "scratch limit" in str(e.value)
    big.close()
    sys_, disc, ex = problems.brusselator(N=16)
    small = Plan(lower(sys_.to_spec(disc)))
    with pytest.raises(L.MolError) as e:
        small.step_ssprk33_noalloc(np.zeros(small.n), 1e-9, 1)
    assert e.value.status == -1 and "device memory" in str(e.value)
    ud = torch.zeros(small.n, dtype=torch.float64, device="cuda")
    for t0, dt in ((0.0, float("inf")), (float("-inf"), 1e-9), (float("nan"), 1e-9)):
        with pytest.raises(L.MolError) as e:
            small.step_ssprk33_noalloc(ud, dt, 1, t0=t0)
        assert e.value.status == -1
    small.close()
