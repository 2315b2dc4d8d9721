"""The reference's compiled f! with its constant folding, against the golden compiled code
(docs/src/generated/bruss_code.md, extracted by tests/golden/make_golden.py), and what the
folding costs in accuracy at the configuration's 1024^2 grid."""
import json
import os

import numpy as np
import pytest

from molgpu import lower, problems
from oracle.folded import brusselator_folded, eval_folded
from oracle.mol_oracle import OracleProblem

GOLD = os.path.join(os.path.dirname(__file__), "golden", "brusselator_dx025_compiled.json")


def _gold():
    with open(GOLD) as fh:
        return json.load(fh)


def _flatten(tree, names):
    """(constant, [(coef, unknown)...] in printed order, product sign) of one compiled output."""
    terms = []

    def walk(t):
        if t[0] == "+":
            walk(t[1])
            walk(t[2])
        else:
            terms.append(t)

    walk(tree)
    const, lin, sq = 0.0, [], None
    for t in terms:
        if t[0] == "num":
            const = t[1]
        elif t[0] == "*" and t[1][0] == "num" and t[2][0] == "var":
            lin.append((t[1][1], names[tuple(t[2][1:])]))
        else:   # (u^2) * v, or ((-1.0) * u^2) * v
            sq = -1.0 if t[1][0] == "*" else 1.0
    return const, lin, sq


def _eval_tree(t, x, names):
    k = t[0]
    if k == "num":
        return t[1]
    if k == "var":
        return x[names[tuple(t[1:])]]
    a, b = _eval_tree(t[1], x, names), _eval_tree(t[2], x, names)
    if k == "+":
        return a + b
    if k == "*":
        return a * b
    assert k == "^" and b == 2.0
    return a * a


@pytest.fixture(scope="module")
def case():
    gold = _gold()
    sys_, disc, _ = problems.brusselator(N=4, forcing=False)
    spec = sys_.to_spec(disc)
    orc = OracleProblem(spec)
    names = {tuple(u): k for k, u in enumerate(gold["unknowns"])}
    return gold, orc, names, brusselator_folded(orc, gold["alpha"])


def test_unknown_order_is_the_reference_argument_order(case):
    gold, orc, names, _ = case
    assert orc.n_unknowns == len(gold["unknowns"]) == 32
    # x fastest within a field, fields u then v (bruss_code.md's argument vector)
    for (f, i, j), k in names.items():
        assert k == orc.offset[f] + (i - 2) + 4 * (j - 2)


def test_folded_coefficients_equal_the_compiled_ones(case):
    """Every coefficient of the compiled f! (160, -644.4, -640, 3.4) is the folding rule's value
    exactly, unknown by unknown, and nothing else appears."""
    gold, orc, names, rows = case
    for i, tree in enumerate(gold["outputs"]):
        const, lin, sq = _flatten(tree, names)
        r = rows[i]
        assert const == r["const"] and sq == r["sq_sign"]
        assert {k: c for c, k in lin} == r["coef"], i
        assert len(lin) == len(r["coef"])


def test_folded_evaluation_equals_the_compiled_code(case):
    """The compiled expressions evaluated in their printed order equal the restated folded form
    summed in the same order bit for bit, and the unfolded oracle to rounding."""
    gold, orc, names, rows = case
    rng = np.random.default_rng(4)
    for _ in range(3):
        x = rng.uniform(0.2, 3.0, size=32)
        ref = np.array([_eval_tree(t, x, names) for t in gold["outputs"]])
        order = [[k for _, k in _flatten(t, names)[1]] for t in gold["outputs"]]
        assert np.array_equal(eval_folded(rows, x, order), ref)
        assert np.linalg.norm(orc.rhs(x, 0.0) - ref) <= 1e-14 * np.linalg.norm(ref)


def test_folding_costs_accuracy_at_1024():
    """At 1024^2 (1/dx^2 = 2^20, alpha = 10) the folded sum cancels terms of ~1e8 down to a
    result of ~1e3: the folded form is ~1e-11 away from the exact semi-discrete RHS whatever
    its summation order, while the per-dimension stencil with power-of-two weights that the
    oracle (and the GPU) evaluates stays ~1e-13 away.  The parity bars therefore use the
    per-dimension form."""
    sys_, disc, _ = problems.brusselator(N=1024, forcing=False)
    lw = lower(sys_.to_spec(disc))
    n = 1024
    u = lw.u0[: n * n].reshape(n, n, order="F")
    v = lw.u0[n * n:].reshape(n, n, order="F")
    orc = OracleProblem(sys_.to_spec(disc))
    w = list(orc.op("centered", 0, 2).stencil_coefs)
    alpha = 10.0
    ld = np.longdouble
    nb = [np.roll(u, 1, 0), np.roll(u, -1, 0), np.roll(u, 1, 1), np.roll(u, -1, 1)]
    exact = (1.0 + ld(1) * u * u * v - ld(4.4) * u
             + ld(alpha) * ld(w[0]) * (ld(1) * nb[0] + nb[1] + nb[2] + nb[3] - 4 * ld(1) * u))
    unfolded = orc.rhs(lw.u0, 0.0)[: n * n].reshape(n, n, order="F")
    c_nb = alpha * w[0]
    c_c = (alpha * w[1] + alpha * w[1]) + -4.4
    folded = ((((1.0 + c_nb * nb[0]) + c_nb * nb[1]) + c_c * u) + c_nb * nb[2]) + c_nb * nb[3]
    folded = folded + (u * u) * v

    def err(a):
        return float(np.linalg.norm((a.astype(ld) - exact)) / np.linalg.norm(exact))

    assert err(unfolded) < 1e-12
    assert err(folded) > 10 * err(unfolded)
