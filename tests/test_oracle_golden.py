"""The oracle against the reference's own known answers (CPU only).

Golden data: tests/golden/*.json, extracted from the reference's test files and
generated docs by tests/golden/make_golden.py.
"""
import json
import math
import os

import numpy as np
import pytest

from oracle import fornberg as OF
from oracle.integrators import TSIT5_A, TSIT5_BTILDE, TSIT5_C, ssprk33, tsit5
from oracle.mol_oracle import OracleProblem, julia_float_range, wrap_periodic

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as fh:
        return json.load(fh)


@pytest.mark.parametrize("case", _load("reference_known_answers.json")["fornberg"])
def test_fornberg_exact(case):
    # test/Components/MOLfornberg_weights.jl: exact equality
    w = OF.calculate_weights(case["order"], case["x0"], case["x"])
    assert w == case["expected"]


@pytest.mark.parametrize("case", _load("reference_known_answers.json")["centered_stencils"])
def test_centered_stencils(case):
    # test/shared/finite_diff_schemes.jl:22-30 (dx = 1)
    D = OF.complete_centered_difference(case["derivative_order"], case["approx_order"], 1.0)
    assert np.allclose(D.stencil_coefs, case["stencil"], rtol=1e-14, atol=1e-15)
    assert len(D.stencil_coefs) == len(case["stencil"])


@pytest.mark.parametrize("case", _load("reference_known_answers.json")["periodic_wrap"])
def test_periodic_wrap(case):
    # test/Components/utils_test.jl:129-137
    I = list(case["I"])
    j = case["j"] - 1
    I[j] = wrap_periodic(I[j], case["l"])
    assert I == case["expected"]


def test_brusselator_generated_equations():
    """The oracle RHS equals the reference's generated ODE system (dx = dy = 1/4)."""
    from molgpu import problems
    g = _load("brusselator_dx025_equations.json")
    sys_, disc, _ = problems.brusselator(N=4, forcing=False)
    orc = OracleProblem(sys_.to_spec(disc))
    assert orc.n_unknowns == 32 == len(g["equations"])
    rng = np.random.default_rng(3)
    u = rng.uniform(0.5, 2.0, orc.n_unknowns)

    def idx(f, i, j):
        return (0 if f == "u" else 16) + (i - 2) + 4 * (j - 2)

    ref = np.zeros(32)
    for e in g["equations"]:
        acc = 0.0
        for term in e["terms"]:
            if term["kind"] == "const":
                acc += term["value"]
            elif term["kind"] == "lin":
                acc += term["coef"] * u[idx(*term["var"])]
            else:
                a = u[idx(*term["a"])]
                acc += term["sign"] * (a * a) * u[idx(*term["b"])]
        ref[idx(*e["lhs"])] = acc
    du = orc.rhs(u, 0.0)
    assert np.allclose(du, ref, rtol=1e-14, atol=1e-12)


def test_brusselator_loop_rhs():
    """Independent loop RHS of test/Brusselator/brusselator_eq.jl:80-105 (periodic 5-point)."""
    from molgpu import problems
    N = 8
    sys_, disc, _ = problems.brusselator(N=N)
    orc = OracleProblem(sys_.to_spec(disc))
    rng = np.random.default_rng(4)
    u = rng.uniform(0.5, 2.0, orc.n_unknowns)
    t = 2.0
    dx = 1.0 / N
    U = u[:N * N].reshape((N, N), order="F")
    V = u[N * N:].reshape((N, N), order="F")
    # unknown index k (0-based) is grid point k+2, i.e. coordinate (k+1)*dx
    xs = (np.arange(N) + 1) * dx
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    f = ((((X - 0.3) ** 2 + (Y - 0.6) ** 2) <= 0.1 ** 2) * (t >= 1.1)) * 5.0
    alpha = 10.0 / dx ** 2
    lap = lambda W: np.roll(W, 1, 0) + np.roll(W, -1, 0) + np.roll(W, 1, 1) + np.roll(W, -1, 1) - 4 * W
    du = alpha * lap(U) + 1.0 + U ** 2 * V - 4.4 * U + f
    dv = alpha * lap(V) + 3.4 * U - U ** 2 * V
    ref = np.concatenate([du.reshape(-1, order="F"), dv.reshape(-1, order="F")])
    assert np.allclose(orc.rhs(u, t), ref, rtol=1e-12, atol=1e-9)


def test_heat_exact_semidiscrete():
    """u0 = sin(pi x) is an eigenvector of the Dirichlet 3-point Laplacian: exact decay exp(lam t)."""
    from molgpu import problems
    sys_, disc, _ = problems.heat1d(n=101)
    orc = OracleProblem(sys_.to_spec(disc))
    u0 = orc.initial_condition()
    dx = 0.01
    lam = -(4 / dx ** 2) * math.sin(math.pi * dx / 2) ** 2
    u, st = tsit5(lambda v, t: orc.rhs(v, t), u0, 0.0, 0.1, 1e-10, 1e-10)
    ref = math.exp(lam * 0.1) * u0
    assert np.max(np.abs(u - ref)) < 1e-9
    # and the PDE's exact solution within the O(dx^2) discretisation error (reference tolerance 0.01)
    x = orc.grid[0][1:-1]
    assert np.max(np.abs(u - np.exp(-math.pi ** 2 * 0.1) * np.sin(math.pi * x))) < 1e-4


def test_tsit5_tableau_order_conditions():
    b = np.array(TSIT5_A[6] + [0.0])
    c = np.array(TSIT5_C)
    for i in range(1, 7):
        assert abs(sum(TSIT5_A[i]) - c[i]) < 1e-14
    for q in range(5):
        assert abs(np.sum(b * c ** q) - 1.0 / (q + 1)) < 1e-13
    assert abs(sum(TSIT5_BTILDE)) < 1e-14


def test_nonlinear_laplacian_unit_coefficient_is_centered():
    """test/shared/finite_diff_schemes.jl:99-143: Dx(1*Dx(u)) discretises to the centered Dxx."""
    from molgpu.symbolic import Differential, Eq, Field, Interval, IV, PDESystem, sin
    from molgpu.api import MOLFiniteDifference
    x, t = IV("x"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    bcs = [Eq(u(x, 0.0), sin(x)), Eq(u(0.0, t), 0.0), Eq(u(20.0, t), 0.0)]
    dom = [(t, Interval(0.0, 1.0)), (x, Interval(0.0, 20.0))]
    disc = MOLFiniteDifference({x: 1.0}, t)
    a = OracleProblem(PDESystem([Eq(Dt(u(x, t)), Dx(1.0 * Dx(u(x, t))))], bcs, dom, [t, x], [u(x, t)]).to_spec(disc))
    b = OracleProblem(PDESystem([Eq(Dt(u(x, t)), Dxx(u(x, t)))], bcs, dom, [t, x], [u(x, t)]).to_spec(disc))
    v = np.random.default_rng(5).standard_normal(a.n_unknowns)
    assert np.allclose(a.rhs(v, 0.0), b.rhs(v, 0.0), rtol=1e-13, atol=1e-13)


def test_julia_ranges():
    g = julia_float_range(0.0, 0.01, 1.0)
    assert len(g) == 101 and g[-1] == 1.0 and g[37] == 0.37
    g = julia_float_range(0.0, 2 * math.pi / 64, 2 * math.pi)
    assert len(g) == 65 and g[-1] == 2 * math.pi


def test_ssprk33_linear_exactness():
    """SSPRK33 applied to u' = lam u equals the degree-3 Taylor polynomial of exp(lam dt)."""
    lam, dt = -0.7, 0.05
    u, _ = ssprk33(lambda v, t: lam * v, np.array([1.0]), 0.0, dt, 1)
    z = lam * dt
    assert abs(u[0] - (1 + z + z * z / 2 + z ** 3 / 6)) < 1e-15
