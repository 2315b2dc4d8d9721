"""Slab decomposition along the slowest dimension (molgpu.slabs) on the CPU: two gloo ranks
exchanging halo planes over torch.distributed, the right-hand side of each rank's local
problem evaluated by the descriptor model of the kernels (tests/desc_interp.py), against the
undivided problem.  The GPU form (local plans, one GPU) is in test_gpu_slabs.py."""
import os
import socket

import numpy as np
import pytest

from molgpu import lower, problems
from molgpu.slabs import Slab

CASES = [("adr3d", dict(N=6, nz_pts=9)), ("brusselator", dict(N=10)), ("burgers", dict(npts=65))]


def _problem(name, kw):
    s, d, ex = getattr(problems, name)(**kw)
    return lower(s.to_spec(d)), ex.get("dt", ex.get("dt_ssprk"))


def _reference(lw, dt, nsteps):
    from desc_interp import DescInterp
    from oracle.integrators import ssprk33
    G = DescInterp(lw)
    ref, _ = ssprk33(lambda v, t: G.rhs(v, t), lw.u0, 0.0, dt, nsteps)
    return ref


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, name, kw, nsteps, out_path):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "methodoflines.jl_gb300"), os.path.join(root, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch
    import torch.distributed as dist
    from desc_interp import DescInterp
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lw, dt = _problem(name, kw)
    sl = Slab(lw, rank, world)
    interp = DescInterp(sl.local)

    def rhs(k, u, t):
        k.copy_(torch.from_numpy(interp.rhs(u.numpy(), t)))

    u = torch.tensor(sl.local.u0)
    sl.ssprk33(u, dt, nsteps, rhs)
    mine = torch.tensor(np.ascontiguousarray(sl.owned(u.numpy())))
    parts = [torch.zeros((len(lw.fields), b - a, sl.plane), dtype=torch.float64)
             for a, b in zip(sl.bounds[:-1], sl.bounds[1:])]
    dist.all_gather(parts, mine) if all(p.shape == mine.shape for p in parts) else _gather_uneven(dist, parts, mine, rank)
    if rank == 0:
        np.save(out_path, torch.cat(parts, dim=1).reshape(-1).numpy())
    dist.barrier()
    dist.destroy_process_group()


def _gather_uneven(dist, parts, mine, rank):
    for r, p in enumerate(parts):
        if r == rank:
            p.copy_(mine)
        dist.broadcast(p, src=r)


def test_slab_geometry_and_local_problem():
    lw, _ = _problem("adr3d", dict(N=6, nz_pts=9))
    sls = [Slab(lw, r, 3) for r in range(3)]
    assert [s.nloc for s in sls] == [2, 2, 3] and sum(s.nloc for s in sls) == 7
    for s in sls:
        assert s.h == 1 and not s.periodic
        assert s.local.npts[2] == s.nloc + 2 + 1 and s.local.lower[2] == 1 and s.local.upper[2] == 0
        assert s.local.n_unknowns == lw.n_unknowns // 7 * (s.nloc + 2)
    # the owned planes of the local initial states are the global initial state
    got = np.concatenate([s.owned(s.local.u0) for s in sls], axis=1).reshape(-1)
    assert np.array_equal(got, lw.u0)
    # bounded ends: the ghost plane beyond the Dirichlet row holds its value (0)
    assert np.all(sls[0].local.u0.reshape(1, 4, 36)[:, 0, :] == 0.0)


def test_unsupported_slabs_refused():
    s, d, _ = problems.nonlinear_diffusion(9, 1.0, 1000)          # Neumann rows along y
    with pytest.raises(NotImplementedError):
        Slab(lower(s.to_spec(d)), 0, 2)
    lw, _ = _problem("brusselator", dict(N=4))
    with pytest.raises(ValueError):
        Slab(lw, 0, 8)                                              # slabs thinner than the halo


@pytest.mark.parametrize("name,kw", CASES)
def test_in_process_slabs_match_undivided(name, kw):
    torch = pytest.importorskip("torch")
    from desc_interp import DescInterp
    lw, dt = _problem(name, kw)
    world, nsteps = 3, 3
    sls = [Slab(lw, r, world) for r in range(world)]
    interps = [DescInterp(s.local) for s in sls]
    us = [torch.tensor(s.local.u0) for s in sls]

    def ex(states):
        Slab.exchange_in_process(sls, states)

    t = 0.0
    for _ in range(nsteps):
        ex(us)
        k = [torch.tensor(interps[r].rhs(us[r].numpy(), t)) for r in range(world)]
        u1 = [us[r] + dt * k[r] for r in range(world)]
        ex(u1)
        k = [torch.tensor(interps[r].rhs(u1[r].numpy(), t + dt)) for r in range(world)]
        u2 = [((3.0 * us[r] + u1[r]) + dt * k[r]) * 0.25 for r in range(world)]
        ex(u2)
        k = [torch.tensor(interps[r].rhs(u2[r].numpy(), t + dt / 2)) for r in range(world)]
        us = [((us[r] + 2.0 * u2[r]) + (2.0 * dt) * k[r]) / 3.0 for r in range(world)]
        t += dt
    got = np.concatenate([s.owned(us[r].numpy()) for r, s in enumerate(sls)], axis=1).reshape(-1)
    ref = _reference(lw, dt, nsteps)
    assert np.linalg.norm(got - ref) <= 1e-14 * np.linalg.norm(ref)


@pytest.mark.parametrize("name,kw", CASES)
def test_two_gloo_ranks_match_undivided(name, kw, tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    nsteps = 3
    out = str(tmp_path / "slabs.npy")
    mp.start_processes(_rank_main, args=(2, _free_port(), name, kw, nsteps, out), nprocs=2, join=True,
                       start_method="spawn")
    lw, dt = _problem(name, kw)
    got = np.load(out)
    ref = _reference(lw, dt, nsteps)
    assert np.linalg.norm(got - ref) <= 1e-14 * np.linalg.norm(ref)
