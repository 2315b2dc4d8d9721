"""Edge-aligned grids on the GPU against the oracle: face rows solved for the ghost points
(generate_bc_eqs.jl:80-160) in the generated code and the interpreter, fixed SSPRK33
trajectories, Tsit5 against the exact solution, the discrete adjoint, Float32 state."""
import math

import numpy as np
import pytest

from molgpu import Plan, lower, problems
from molgpu import _lib as L
from oracle.integrators import ssprk33, tsit5
from oracle.mol_oracle import OracleProblem

pytestmark = pytest.mark.gpu

CASES = {
    "neumann_o2": lambda: problems.neumann_cosine_edge(dx=0.005, order=2),
    "neumann_o8": lambda: problems.neumann_cosine_edge(dx=0.005, order=8),
    "robin_2d": lambda: problems.robin_2d_edge(),
}


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _setup(name):
    s, d, ex = CASES[name]()
    spec = s.to_spec(d)
    return spec, lower(spec), OracleProblem(spec), ex


@pytest.mark.parametrize("name", sorted(CASES))
def test_edge_rhs_and_trajectory(gpu_lib, name):
    spec, lw, orc, ex = _setup(name)
    plan = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(plan.handle) == 1
    v = lw.u0 + 0.05 * np.random.default_rng(4).standard_normal(lw.n_unknowns)
    for t in (0.0, 0.37):
        du = np.zeros(lw.n_unknowns)
        plan.rhs(du, v, None, t)
        ref = orc.rhs(v, t)
        assert _rel(du, ref) <= 1e-12, (name, t)
    u = lw.u0.copy()
    plan.step_ssprk33(u, ex["dt"], 40, t0=0.1)
    ref, _ = ssprk33(lambda w, tt: orc.rhs(w, tt), lw.u0, 0.1, ex["dt"], 40)
    assert _rel(u, ref) <= 1e-10, name
    plan.close()


@pytest.mark.parametrize("name", ["neumann_o8", "robin_2d"])
def test_edge_generated_matches_interpreter(gpu_lib, name, monkeypatch):
    spec, lw, orc, ex = _setup(name)
    gen = Plan(lw)
    monkeypatch.setenv("MOL_DISABLE_CODEGEN", "1")
    interp = Plan(lw)
    assert L.lib().mol_plan_uses_codegen(interp.handle) == 0
    u = lw.u0 * 1.01
    a, b = np.zeros_like(u), np.zeros_like(u)
    gen.rhs(a, u, None, 0.9)
    interp.rhs(b, u, None, 0.9)
    assert _rel(a, b) < 1e-13
    x, y = lw.u0.copy(), lw.u0.copy()
    gen.step_ssprk33(x, ex["dt"], 20)
    interp.step_ssprk33(y, ex["dt"], 20)
    assert _rel(x, y) < 1e-12


def test_edge_neumann_tsit5_exact(gpu_lib):
    """The reference's Test 03 on an edge-aligned grid (order 8, u_x = 0 at both faces):
    the solve tracks exp(-pi^2 t) cos(pi x) and the oracle's Tsit5."""
    s, d, _ = problems.neumann_cosine_edge(dx=0.02, order=8)
    spec = s.to_spec(d)
    lw, orc = lower(spec), OracleProblem(spec)
    plan = Plan(lw)
    u = lw.u0.copy()
    st = plan.solve_tsit5(u, 0.0, 0.1, 1e-10, 1e-10)
    ref, rst = tsit5(lambda v, t: orc.rhs(v, t), lw.u0, 0.0, 0.1, 1e-10, 1e-10)
    assert _rel(u, ref) < 1e-9
    assert abs(st["naccept"] - rst["naccept"]) <= 2
    xs = lw.grids[0][1:-1]
    assert np.max(np.abs(u - math.exp(-math.pi ** 2 * 0.1) * np.cos(math.pi * xs))) < 1e-7
    plan.close()


def test_edge_adjoint_matches_finite_differences(gpu_lib):
    spec, lw, orc, ex = _setup("robin_2d")
    plan = Plan(lw)
    dt, n = ex["dt"], 25
    target = np.zeros(lw.n_unknowns)

    def loss(u0):
        u = u0.copy()
        plan.step_ssprk33(u, dt, n, t0=0.0)
        return 0.5 * float(np.sum((u - target) ** 2))

    g = np.zeros(lw.n_unknowns)
    plan.adjoint_ssprk33(lw.u0, dt, n, target, nsnap=4, dLdu0=g)
    w = np.random.default_rng(9).standard_normal(lw.n_unknowns)

    def cd(h):
        return (loss(lw.u0 + h * w) - loss(lw.u0 - h * w)) / (2 * h)

    fd = (4.0 * cd(5e-7) - cd(1e-6)) / 3.0
    assert abs(g @ w - fd) <= 1e-6 * abs(fd), (g @ w, fd)
    plan.close()


def test_edge_f32state(gpu_lib):
    spec, lw, orc, ex = _setup("robin_2d")
    plan = Plan(lw)
    u64 = lw.u0.copy()
    u32 = u64.astype(np.float32)
    plan.step_ssprk33(u64, ex["dt"], 20)
    plan.step_ssprk33(u32, ex["dt"], 20)
    assert _rel(u32.astype(np.float64), u64) < 1e-5
    plan.close()
