"""Extract the reference's own known answers into ``tests/golden/*.json``.

MethodOfLines.jl is Julia and cannot run here, so its golden vectors are read
as text from its test files and generated documentation:

* ``test/Components/MOLfornberg_weights.jl:4-30``  exact Fornberg weights
* ``test/shared/finite_diff_schemes.jl:22-30``     centered stencils, orders 2 and 4
* ``test/Components/utils_test.jl:129-137``        periodic index wrap
* ``docs/src/generated/bruss_ode_eqs.md``          the generated Brusselator ODE system
  at dx = dy = 1/4 (the reference's own discretisation, after ModelingToolkit)
* ``docs/src/generated/bruss_code.md``             the compiled f! of the same system: its
  argument order and each output's expression with the folded coefficients

Usage: ``python tests/golden/make_golden.py [REFERENCE_ROOT]``.  The JSON files are
committed so the tests never need the reference checkout.
"""
from __future__ import annotations

import json
import os
import re
import sys
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))


def _num(s: str) -> float:
    s = s.strip()
    if "/" in s:
        a, b = s.split("/")
        return float(Fraction(int(a.strip()), int(b.strip())))
    return float(s)


def fornberg_cases(root):
    txt = open(os.path.join(root, "test/Components/MOLfornberg_weights.jl")).read()
    cases = []
    pat = re.compile(
        r"order\s*=\s*(\d+)\s*\n\s*z\s*=\s*([-\d.]+)\s*\n\s*x\s*=\s*(\[[^\]]*\]|collect\([^)]*\))\s*\n"
        r"\s*@test MethodOfLines\.calculate_weights\(order, z, x\) ==\s*\n?\s*\[([^\]]*)\]")
    for m in pat.finditer(txt):
        order = int(m.group(1))
        z = float(m.group(2))
        xs = m.group(3)
        if xs.startswith("collect"):
            a, b = re.findall(r"(-?\d+):(-?\d+)", xs)[0]
            x = list(range(int(a), int(b) + 1))
        else:
            x = [_num(v) for v in xs.strip("[]").split(",")]
        expected = [_num(v) for v in m.group(4).split(",")]
        cases.append({"order": order, "x0": z, "x": x, "expected": expected,
                      "source": "test/Components/MOLfornberg_weights.jl"})
    return cases


def centered_lists(root):
    txt = open(os.path.join(root, "test/shared/finite_diff_schemes.jl")).read()
    m = re.search(r"weights = \[\]\s*\n(.*?)for d in 1:3", txt, re.S)
    block = m.group(1)
    lists = re.findall(r"\[([^\[\]]+)\]", block)
    vals = [[_num(v) for v in l.split(",")] for l in lists]
    # two push! calls, each a (d=1, d=2, d=3) tuple, for approx_order 2 then 4
    out = []
    for k, p in enumerate((2, 4)):
        for d in (1, 2, 3):
            out.append({"approx_order": p, "derivative_order": d, "dx": 1.0,
                        "stencil": vals[3 * k + d - 1],
                        "source": "test/shared/finite_diff_schemes.jl:22-30"})
    return out


def wrap_cases(root):
    txt = open(os.path.join(root, "test/Components/utils_test.jl")).read()
    m = re.search(r'@testset "Periodic Wraparound" begin(.*?)\nend', txt, re.S)
    out = []
    for I, args, R in re.findall(
            r"I = CartesianIndex\(([^)]*)\)\s*\n\s*@test MethodOfLines\._wrapperiodic\(I, ([^)]*)\) == CartesianIndex\(([^)]*)\)",
            m.group(1)):
        N, j, l = [int(v) for v in args.split(",")]
        out.append({"I": [int(v) for v in I.split(",")], "N": N, "j": j, "l": l,
                    "expected": [int(v) for v in R.split(",")],
                    "source": "test/Components/utils_test.jl:129-137"})
    return out


_TERM = re.compile(r"\s*([+-])?\s*(\([^()]*\([^()]*\)\^2\)\*[uv]\[\d+, \d+\]\(t\)|[\d.]+[uv]\[\d+, \d+\]\(t\)|[\d.]+)")


def brusselator_equations(root):
    txt = open(os.path.join(root, "docs/src/generated/bruss_ode_eqs.md")).read()
    eqs = []
    for line in txt.splitlines():
        line = line.strip().lstrip("[").rstrip(",").rstrip("]").strip()
        m = re.match(r"Differential\(t\)\(([uv])\[(\d+), (\d+)\]\(t\)\) ~ (.*)$", line)
        if not m:
            continue
        f, i, j, rhs = m.group(1), int(m.group(2)), int(m.group(3)), m.group(4).rstrip(",").strip()
        terms = []
        pos = 0
        while pos < len(rhs):
            t = _TERM.match(rhs, pos)
            if not t:
                raise ValueError(f"cannot parse {rhs[pos:]!r}")
            sign = -1.0 if t.group(1) == "-" else 1.0
            body = t.group(2)
            pm = re.match(r"\(\(([uv])\[(\d+), (\d+)\]\(t\)\^2\)\)\*([uv])\[(\d+), (\d+)\]\(t\)", body) or \
                re.match(r"\(([uv])\[(\d+), (\d+)\]\(t\)\^2\)\*([uv])\[(\d+), (\d+)\]\(t\)", body)
            lm = re.match(r"([\d.]+)([uv])\[(\d+), (\d+)\]\(t\)", body)
            if pm:
                terms.append({"kind": "sq_times", "sign": sign,
                              "a": [pm.group(1), int(pm.group(2)), int(pm.group(3))],
                              "b": [pm.group(4), int(pm.group(5)), int(pm.group(6))]})
            elif lm:
                terms.append({"kind": "lin", "coef": sign * float(lm.group(1)),
                              "var": [lm.group(2), int(lm.group(3)), int(lm.group(4))]})
            else:
                terms.append({"kind": "const", "value": sign * float(body)})
            pos = t.end()
        eqs.append({"lhs": [f, i, j], "terms": terms})
    return {"dx": 0.25, "alpha": 10.0, "source": "docs/src/generated/bruss_ode_eqs.md", "equations": eqs}


def _parse_prefix(s: str, pos: int):
    """One Julia prefix-call expression of the generated code: ``(+)(a, b)``, ``(*)(a, b)``,
    ``(^)(x, 2)``, a number or ``var"u[i, j](t)"``; returns (tree, next position)."""
    while s[pos] == " ":
        pos += 1
    if s.startswith('var"', pos):
        end = s.index('"', pos + 4)
        m = re.match(r"([uv])\[(\d+), (\d+)\]\(t\)", s[pos + 4:end])
        return ["var", m.group(1), int(m.group(2)), int(m.group(3))], end + 1
    if s[pos] == "(" and s[pos + 2] == ")" and s[pos + 1] in "+*^":
        op = s[pos + 1]
        pos += 3
        assert s[pos] == "("
        pos += 1
        args = []
        while True:
            a, pos = _parse_prefix(s, pos)
            args.append(a)
            while s[pos] == " ":
                pos += 1
            if s[pos] == ",":
                pos += 1
                continue
            assert s[pos] == ")", s[pos:pos + 20]
            return [op] + args, pos + 1
    m = re.match(r"-?[\d.]+(e-?\d+)?", s[pos:])
    return ["num", float(m.group(0))], pos + m.end()


def brusselator_compiled(root):
    """The compiled f! at dx = dy = 1/4 (docs/src/generated/bruss_code.md): the unknown order
    of its argument vector and, for every output, the expression tree with its folded
    coefficients (alpha/dx^2 in every tap, centre coefficients merged) in the printed order."""
    txt = open(os.path.join(root, "docs/src/generated/bruss_code.md")).read()
    start = txt.index("function (ˍ₋out, ˍ₋arg1, ˍ₋arg2, t)")
    body = txt[start:]
    unknowns = []
    for m in re.finditer(r'var"([uv])\[(\d+), (\d+)\]\(t\)" = @inbounds\(ˍ₋arg1\[(\d+)\]\)', body):
        assert int(m.group(4)) == len(unknowns) + 1
        unknowns.append([m.group(1), int(m.group(2)), int(m.group(3))])
    outs = {}
    for m in re.finditer(r"ˍ₋out\[(\d+)\] = ", body):
        tree, _ = _parse_prefix(body, m.end())
        outs[int(m.group(1))] = tree
    return {"dx": 0.25, "alpha": 10.0, "source": "docs/src/generated/bruss_code.md",
            "unknowns": unknowns, "outputs": [outs[k] for k in range(1, len(outs) + 1)]}


def main(root="/root/reference"):
    golden = {
        "fornberg": fornberg_cases(root),
        "centered_stencils": centered_lists(root),
        "periodic_wrap": wrap_cases(root),
    }
    with open(os.path.join(HERE, "reference_known_answers.json"), "w") as fh:
        json.dump(golden, fh, indent=1)
    with open(os.path.join(HERE, "brusselator_dx025_equations.json"), "w") as fh:
        json.dump(brusselator_equations(root), fh, indent=1)
    with open(os.path.join(HERE, "brusselator_dx025_compiled.json"), "w") as fh:
        json.dump(brusselator_compiled(root), fh)
    print("fornberg", len(golden["fornberg"]), "stencils", len(golden["centered_stencils"]),
          "wrap", len(golden["periodic_wrap"]))


if __name__ == "__main__":
    main(*sys.argv[1:])
