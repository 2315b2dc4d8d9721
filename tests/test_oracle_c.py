"""The oracle's C/OpenMP restatement of the headline workload (oracle/c/bruss_oracle.c)
against the numpy oracle: the RHS before and after the forcing switches on, and fixed
SSPRK33 trajectories, on one and on several threads."""
import numpy as np
import pytest

from molgpu import lower, problems
from oracle.c_port import Brusselator
from oracle.integrators import ssprk33
from oracle.mol_oracle import OracleProblem


@pytest.mark.parametrize("N", [8, 32])
def test_c_port_rhs_matches_numpy_oracle(N):
    sys_, disc, _ = problems.brusselator(N=N)
    spec = sys_.to_spec(disc)
    lw = lower(spec)
    b, orc = Brusselator(lw), OracleProblem(spec)
    u = lw.u0 + 0.1 * np.random.default_rng(N).standard_normal(lw.n_unknowns)
    for t in (0.5, 1.2):
        ref = orc.rhs(u, t)
        assert np.max(np.abs(b.rhs(u, t) - ref)) <= 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("nthreads", [1, 0])
def test_c_port_ssprk33_matches_numpy_oracle(nthreads):
    sys_, disc, ex = problems.brusselator(N=32)
    spec = sys_.to_spec(disc)
    lw = lower(spec)
    b, orc = Brusselator(lw), OracleProblem(spec)
    got = b.ssprk33(lw.u0, 1.0, ex["dt_ssprk"], 25, nthreads)
    ref, _ = ssprk33(lambda v, t: orc.rhs(v, t), lw.u0, 1.0, ex["dt_ssprk"], 25)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


@pytest.mark.parametrize("N,nz", [(8, 10), (12, 11)])
def test_c_port_adr_rhs_matches_numpy_oracle(N, nz):
    """The 3-D advection-diffusion-reaction restatement (oracle/c/adr_oracle.c) against the
    numpy oracle's general evaluation of the same system."""
    from oracle.c_port import ADR3D
    sys_, disc, _ = problems.adr3d(N=N, nz_pts=nz)
    spec = sys_.to_spec(disc)
    lw = lower(spec)
    a, orc = ADR3D(lw), OracleProblem(spec)
    u = lw.u0 + 0.05 * np.random.default_rng(N).standard_normal(lw.n_unknowns)
    ref = orc.rhs(u, 0.1)
    got = a.rhs(u)
    assert np.linalg.norm(got - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("nthreads", [1, 0])
def test_c_port_adr_ssprk33_matches_numpy_oracle(nthreads):
    from oracle.c_port import ADR3D
    sys_, disc, ex = problems.adr3d(N=8, nz_pts=10)
    spec = sys_.to_spec(disc)
    lw = lower(spec)
    a, orc = ADR3D(lw), OracleProblem(spec)
    dt = ex["dt"]
    got = a.ssprk33(lw.u0, dt, 12, nthreads)
    ref, _ = ssprk33(lambda v, t: orc.rhs(v, t), lw.u0, 0.0, dt, 12)
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)
