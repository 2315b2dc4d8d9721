"""The reference's compiled right-hand side of the Brusselator, restated with its constant
folding (test infrastructure, like the rest of ``oracle/``).

MethodOfLines emits, per unknown, the generated equation with every derivative replaced by
its stencil: alpha*(Dxx u + Dyy u) becomes, on the periodic grid, the taps of each
dimension's centered second derivative (1/dx^2)[1, -2, 1] times alpha
(docs/src/generated/bruss_ode_eqs.md: ``1.0 + 160.0u[3, 2] + 160.0u[5, 2] - 320.0u[2, 2] +
160.0u[2, 3] + 160.0u[2, 5] - 320.0u[2, 2] + (u[2, 2]^2)*v[2, 2] - 4.4u[2, 2]``).
ModelingToolkit compiles that into f! (src/MOL_discretization.jl:171-201;
docs/src/generated/bruss_code.md:82-113) with SymbolicUtils' canonical sums: one
coefficient per distinct unknown, alpha*w folded into every tap and the coefficients of one
unknown added in the order its terms occur (-320 - 320 - 4.4 = -644.4 at the centre of the
u equation, -640 for v), the constant first and the u^2 v product last.

``brusselator_folded`` restates that rule from the oracle's own stencil tables, and
``eval_folded`` evaluates it.  The order in which SymbolicUtils prints the linear terms of
an output is its own (it is not the order of the unknowns); ``eval_folded`` sums the taps
in the order given, and the tests pin the rule against the compiled f! at dx = 1/4, where
every coefficient is exact and the order does not change the value.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

from .mol_oracle import OracleProblem, central_taps


def _unknown_index(orc: OracleProblem, f: str, idx: Tuple[int, ...]) -> int:
    """Position in the unknown vector of the 1-based grid point idx of field f."""
    shp = orc.shape[f]
    flat = 0
    stride = 1
    for j in range(orc.nd):
        flat += (idx[j] - 1 - orc.lower[f][j]) * stride
        stride *= shp[j]
    return orc.offset[f] + flat


def brusselator_folded(orc: OracleProblem, alpha: float, a_lin: float = -4.4, b_lin: float = 3.4):
    """Per unknown of the periodic Brusselator (fields u, v): the constant, the folded linear
    coefficients {unknown: coefficient} in order of first occurrence, and the sign of the
    u^2 v product, as the compiled f! holds them."""
    assert orc.fields == ["u", "v"] and orc.nd == 2
    n = orc.npts
    ops = [orc.op("centered", j, 2) for j in range(2)]
    rows: List[dict] = []
    for f in ("u", "v"):
        for b in orc.interior_index(f, 1):
            for a in orc.interior_index(f, 0):
                coef: Dict[int, float] = {}
                here = _unknown_index(orc, f, (int(a), int(b)))

                def add(k, c):
                    coef[k] = coef[k] + c if k in coef else c

                if f == "v":      # 3.4 u, then alpha * (Dxx v + Dyy v), then -u^2 v
                    add(_unknown_index(orc, "u", (int(a), int(b))), b_lin)
                for j, D in enumerate(ops):
                    w, taps = central_taps(D, int(a) if j == 0 else int(b), n[j], True)
                    # bruss_ode_eqs.md prints each dimension's neighbours in ascending index
                    # order and then the centre
                    pts = sorted(zip(w, taps), key=lambda wt: (wt[1] == (int(a) if j == 0 else int(b)), wt[1]))
                    for wk, tk in pts:
                        idx = (tk, int(b)) if j == 0 else (int(a), tk)
                        add(_unknown_index(orc, f, idx), alpha * wk)
                if f == "u":      # 1.0 + ... + u^2 v - 4.4 u
                    add(here, a_lin)
                rows.append({"const": 1.0 if f == "u" else 0.0, "coef": coef,
                             "sq_sign": 1.0 if f == "u" else -1.0,
                             "u": _unknown_index(orc, "u", (int(a), int(b))),
                             "v": _unknown_index(orc, "v", (int(a), int(b)))})
    return rows


def eval_folded(rows, x: np.ndarray, order=None) -> np.ndarray:
    """f(x) in the folded form: ((const + c_1 x_1) + c_2 x_2 + ...) + sign u^2 v, the linear
    terms in `order[i]` (a list of unknowns per output) or in their order of occurrence."""
    out = np.empty(len(rows))
    for i, r in enumerate(rows):
        keys = order[i] if order is not None else list(r["coef"].keys())
        acc = r["const"]
        for k in keys:
            acc = acc + r["coef"][k] * x[k]
        uu = x[r["u"]]
        out[i] = acc + (r["sq_sign"] * (uu * uu)) * x[r["v"]]
    return out
