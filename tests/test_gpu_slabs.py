"""Slab decomposition on the GPU: every slab's local problem as its own plan (one GPU, the
slabs of one decomposition held by one process, ghost planes refreshed by tensor copies
between stages), SSPRK33 steps against the undivided plan."""
import numpy as np
import pytest

from molgpu import Plan, lower, problems
from molgpu.slabs import Slab

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,kw,world", [("adr3d", dict(N=32, nz_pts=34), 3), ("brusselator", dict(N=64), 2),
                                           ("burgers", dict(npts=513), 4)])
def test_slabs_match_undivided_plan(gpu_lib, name, kw, world):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    s, d, ex = getattr(problems, name)(**kw)
    lw = lower(s.to_spec(d))
    dt = ex.get("dt", ex.get("dt_ssprk"))
    stream = torch.cuda.current_stream().cuda_stream
    nsteps = 12
    whole = Plan(lw)
    whole.set_stream(stream)
    ref = torch.tensor(lw.u0, device="cuda")
    whole.step_ssprk33(ref, dt, nsteps)
    sls = [Slab(lw, r, world) for r in range(world)]
    plans = [Plan(sl.local) for sl in sls]
    for p in plans:
        p.set_stream(stream)
    us = [torch.tensor(sl.local.u0, device="cuda") for sl in sls]
    ks = [torch.empty_like(u) for u in us]

    def rhs_all(states, t):
        for p, k, u in zip(plans, ks, states):
            p.rhs(k, u, None, t)

    t = 0.0
    for _ in range(nsteps):
        Slab.exchange_in_process(sls, us)
        rhs_all(us, t)
        u1 = [u + dt * k for u, k in zip(us, ks)]
        Slab.exchange_in_process(sls, u1)
        rhs_all(u1, t + dt)
        u2 = [((3.0 * u + a) + dt * k) * 0.25 for u, a, k in zip(us, u1, ks)]
        Slab.exchange_in_process(sls, u2)
        rhs_all(u2, t + dt / 2)
        us = [((u + 2.0 * b) + (2.0 * dt) * k) / 3.0 for u, b, k in zip(us, u2, ks)]
        t += dt
    got = np.concatenate([sl.owned(u.cpu().numpy()) for sl, u in zip(sls, us)], axis=1).reshape(-1)
    want = ref.cpu().numpy()
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
    for p in plans + [whole]:
        p.close()
