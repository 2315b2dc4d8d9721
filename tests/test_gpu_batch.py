"""Batched ensemble: one persistent launch for many uneven instances, against per-instance plans."""
import numpy as np
import pytest

from molgpu import Batch, Plan, lower, problems
from oracle.integrators import ssprk33
from oracle.mol_oracle import OracleProblem

pytestmark = pytest.mark.gpu


def _members(specs):
    lws, dts = [], []
    for n, k, seed in specs:
        sys_, disc, _ = problems.nonlinear_diffusion(n, k, seed)
        lw = lower(sys_.to_spec(disc))
        lws.append(lw)
        dx = 1.0 / (n - 1)
        dts.append(0.125 * dx * dx / float(np.max(lw.u0)) ** 2)
    return lws, np.array(dts)


SPECS = [(9, 1.3, 1000), (33, 0.2, 1001), (5, 1.9, 1002), (17, 0.7, 1003), (40, 1.1, 1004), (12, 0.0, 1005),
         (64, 1.6, 1006)]


def test_batch_matches_individual_plans(gpu_lib):
    lws, dts = _members(SPECS)
    batch = Batch(lws)
    assert batch.offsets[-1] == sum(lw.n_unknowns for lw in lws)
    u = batch.pack([lw.u0 for lw in lws])
    batch.step_ssprk33(u, dts, 25, t0=0.0)
    for i, lw in enumerate(lws):
        ref = lw.u0.copy()
        Plan(lw).step_ssprk33(ref, dts[i], 25, t0=0.0)
        got = u[batch.offsets[i]:batch.offsets[i + 1]]
        assert np.allclose(got, ref, rtol=1e-13, atol=1e-15), i


def test_batch_against_oracle(gpu_lib):
    lws, dts = _members(SPECS[:3])
    batch = Batch(lws)
    u = batch.pack([lw.u0 for lw in lws])
    batch.step_ssprk33(u, dts, 10, t0=0.0)
    for i, (n, k, seed) in enumerate(SPECS[:3]):
        sys_, disc, _ = problems.nonlinear_diffusion(n, k, seed)
        orc = OracleProblem(sys_.to_spec(disc))
        ref, _ = ssprk33(lambda v, t: orc.rhs(v, t), lws[i].u0, 0.0, dts[i], 10)
        got = u[batch.offsets[i]:batch.offsets[i + 1]]
        assert np.linalg.norm(got - ref) <= 1e-10 * np.linalg.norm(ref)


def test_batch_f32state_and_tuning(gpu_lib):
    lws, dts = _members(SPECS)
    batch = Batch(lws)
    u64 = batch.pack([lw.u0 for lw in lws])
    u32 = u64.astype(np.float32)
    batch.tune(128, 2)
    batch.step_ssprk33(u64, dts, 15)
    batch.step_ssprk33(u32, dts, 15)
    err = np.linalg.norm(u32.astype(np.float64) - u64) / np.linalg.norm(u64)
    assert err < 1e-5
    batch.tune()  # back to autotuning
    again = batch.pack([lw.u0 for lw in lws])
    batch.step_ssprk33(again, dts, 15)
    assert np.allclose(again, u64, rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("tile_cells", [-1, 32, 128, 4096])
def test_batch_schedules_agree(gpu_lib, tile_cells):
    """Tiled schedule (instances split over many CTAs, stages ordered by counters) and the
    one-CTA-per-instance schedule give the per-instance plans' trajectories; tiles of 32
    cells split every member here, 4096 leaves each member in one tile."""
    lws, dts = _members(SPECS)
    batch = Batch(lws)
    batch.tune(128, 4, tile_cells)
    u = batch.pack([lw.u0 for lw in lws])
    batch.step_ssprk33(u, dts, 20, t0=0.0)
    batch.check()
    for i, lw in enumerate(lws):
        ref = lw.u0.copy()
        Plan(lw).step_ssprk33(ref, dts[i], 20, t0=0.0)
        got = u[batch.offsets[i]:batch.offsets[i + 1]]
        assert np.allclose(got, ref, rtol=1e-13, atol=1e-15), (tile_cells, i)


def test_batch_tiled_device_arrays_repeat(gpu_lib):
    """Graph replays of the tiled schedule on device arrays reset their counters: two
    runs of 7 steps (the second a replay of the first's graph; the members are
    autonomous, so t0 does not matter) equal one plan run of 14."""
    torch = pytest.importorskip("torch")
    lws, dts = _members(SPECS)
    batch = Batch(lws)
    batch.tune(256, 2, 64)
    st = torch.cuda.Stream()
    batch.set_stream(st.cuda_stream)
    u = torch.tensor(batch.pack([lw.u0 for lw in lws]), device="cuda")
    with torch.cuda.stream(st):
        batch.step_ssprk33(u, dts, 7)
        batch.step_ssprk33(u, dts, 7)
    batch.check()
    got_all = u.cpu().numpy()
    for i, lw in enumerate(lws):
        ref = lw.u0.copy()
        Plan(lw).step_ssprk33(ref, dts[i], 14, t0=0.0)
        got = got_all[batch.offsets[i]:batch.offsets[i + 1]]
        assert np.allclose(got, ref, rtol=1e-13, atol=1e-15), i


def test_batch_bounded_wait_reports_abandoned_run(gpu_lib, monkeypatch):
    """Failure detection without a GPU fault: a dependency that is never met (the host starts
    the ticket after round 0, so round-1 tiles wait for tiles no CTA runs) makes the bounded
    waits run out; every CTA leaves, mol_batch_check reports the abandoned run, and the
    ensemble works normally afterwards."""
    torch = pytest.importorskip("torch")
    from molgpu._lib import MolError
    lws, dts = _members(SPECS)
    batch = Batch(lws)
    batch.tune(128, 2, 64)
    st = torch.cuda.Stream()
    batch.set_stream(st.cuda_stream)
    u = torch.tensor(batch.pack([lw.u0 for lw in lws]), device="cuda")
    monkeypatch.setenv("MOL_BATCH_INJECT_SKIP_ROUND", "1")
    monkeypatch.setenv("MOL_BATCH_SPIN_LIMIT", "2000")
    batch.step_ssprk33(u, dts, 3)
    with pytest.raises(MolError, match="poll budget"):
        batch.check()
    monkeypatch.delenv("MOL_BATCH_INJECT_SKIP_ROUND")
    monkeypatch.delenv("MOL_BATCH_SPIN_LIMIT")
    u = torch.tensor(batch.pack([lw.u0 for lw in lws]), device="cuda")
    batch.step_ssprk33(u, dts, 6)
    batch.check()
    got_all = u.cpu().numpy()
    for i, lw in enumerate(lws):
        ref = lw.u0.copy()
        Plan(lw).step_ssprk33(ref, dts[i], 6, t0=0.0)
        assert np.allclose(got_all[batch.offsets[i]:batch.offsets[i + 1]], ref, rtol=1e-13, atol=1e-15), i


@pytest.mark.parametrize("family", ["stretched", "weno_bounded", "edge"])
def test_batch_members_with_grid_variants(gpu_lib, family):
    """Ensembles of members on nonuniform grids (per-point rows), with WENO on a bounded
    dimension (extrapolated points) and on edge-aligned grids (ghost rows) step like their
    plans."""
    if family == "stretched":
        made = [problems.stretched_reaction_diffusion(n=n, order=4) for n in (41, 97, 200)]
    elif family == "weno_bounded":
        made = [problems.viscous_burgers_weno_bounded(n=n, order=2) for n in (33, 65, 129)]
    else:
        made = [problems.neumann_cosine_edge(dx=dx, order=4) for dx in (0.05, 0.02, 0.01)]
    lws = [lower(s.to_spec(d)) for s, d, _ in made]
    dts = np.array([ex["dt"] for _, _, ex in made])
    batch = Batch(lws)
    batch.tune(128, 2, 64)
    u = batch.pack([lw.u0 for lw in lws])
    batch.step_ssprk33(u, dts, 12, t0=0.0)
    batch.check()
    for i, lw in enumerate(lws):
        ref = lw.u0.copy()
        Plan(lw).step_ssprk33(ref, dts[i], 12, t0=0.0)
        assert np.allclose(u[batch.offsets[i]:batch.offsets[i + 1]], ref, rtol=1e-13, atol=1e-15), (family, i)
