"""A small symbolic layer mirroring the ModelingToolkit/MethodOfLines user API.

Expressions are immutable trees of tuples; ``PDESystem.to_spec`` turns a system
plus ``MOLFiniteDifference`` options into plain data (nested tuples, floats and
strings) that the lowering consumes.

    x, y, t = IV("x"), IV("y"), IV("t")
    u = Field("u")
    Dt, Dx, Dxx = Differential(t), Differential(x), Differential(x) ** 2
    eq = Eq(Dt(u(x, t)), Dxx(u(x, t)))
"""
from __future__ import annotations

import math
from typing import Callable, Dict, List, Sequence


def _tree(v):
    if isinstance(v, Expr):
        return v.t
    if isinstance(v, (int, float)) and not isinstance(v, bool):
        return ("num", float(v))
    if isinstance(v, bool):
        return ("num", 1.0 if v else 0.0)
    raise TypeError(f"cannot use {type(v).__name__} in an expression")


class Expr:
    __slots__ = ("t",)

    def __init__(self, t):
        self.t = t

    def __add__(self, o): return Expr(("add", self.t, _tree(o)))
    def __radd__(self, o): return Expr(("add", _tree(o), self.t))
    def __sub__(self, o): return Expr(("sub", self.t, _tree(o)))
    def __rsub__(self, o): return Expr(("sub", _tree(o), self.t))
    def __mul__(self, o): return Expr(("mul", self.t, _tree(o)))
    def __rmul__(self, o): return Expr(("mul", _tree(o), self.t))
    def __truediv__(self, o): return Expr(("div", self.t, _tree(o)))
    def __rtruediv__(self, o): return Expr(("div", _tree(o), self.t))
    def __pow__(self, o): return Expr(("pow", self.t, _tree(o)))
    def __rpow__(self, o): return Expr(("pow", _tree(o), self.t))
    def __neg__(self): return Expr(("neg", self.t))
    def __pos__(self): return self
    def __le__(self, o): return Expr(("cmp", "<=", self.t, _tree(o)))
    def __lt__(self, o): return Expr(("cmp", "<", self.t, _tree(o)))
    def __ge__(self, o): return Expr(("cmp", ">=", self.t, _tree(o)))
    def __gt__(self, o): return Expr(("cmp", ">", self.t, _tree(o)))
    __hash__ = object.__hash__

    def __repr__(self):
        return f"Expr({self.t!r})"


class IV(Expr):
    """Independent variable (space or time)."""
    __slots__ = ("name",)

    def __init__(self, name: str):
        super().__init__(("iv", name))
        self.name = name


class Param(Expr):
    """A parameter with a default value (part of the ODEProblem's p)."""
    __slots__ = ("name", "default")

    def __init__(self, name: str, default: float):
        super().__init__(("param", name))
        self.name = name
        self.default = float(default)


class Field:
    """A dependent variable u(..); applying it to variables gives an expression."""

    def __init__(self, name: str):
        self.name = name

    def __call__(self, *args):
        return FieldApp(self, args)


class FieldApp(Expr):
    __slots__ = ("field", "args")

    def __init__(self, field: Field, args):
        self.field = field
        self.args = tuple(args)
        if all(isinstance(a, IV) for a in args):
            super().__init__(("field", field.name, tuple(a.name for a in args)))
        else:
            spec = tuple((None if isinstance(a, IV) else float(a)) for a in args)
            super().__init__(("fieldat", field.name, tuple(a.name if isinstance(a, IV) else None for a in args), spec))


class Differential:
    def __init__(self, iv: IV, order: int = 1):
        self.iv = iv
        self.order = int(order)

    def __pow__(self, n: int):
        return Differential(self.iv, self.order * int(n))

    def __call__(self, e):
        t = _tree(e)
        # D(D^k(u)) along the same variable of a plain field is D^(k+1)(u)
        if t[0] == "D" and t[1] == self.iv.name and t[3][0] in ("field", "fieldat"):
            return Expr(("D", self.iv.name, self.order + t[2], t[3]))
        return Expr(("D", self.iv.name, self.order, t))


def _fn(name):
    def f(e):
        if isinstance(e, (int, float)):
            return getattr(math, name)(e) if name != "abs" else abs(e)
        return Expr(("fn", name, _tree(e)))
    f.__name__ = name
    return f


sin, cos, tan, exp, log, sqrt, tanh, sinh, cosh, atan = (
    _fn(n) for n in ("sin", "cos", "tan", "exp", "log", "sqrt", "tanh", "sinh", "cosh", "atan"))
abs_ = _fn("abs")


def ifelse(c, a, b):
    return Expr(("ifelse", _tree(c), _tree(a), _tree(b)))


_REGISTRY: Dict[str, Callable] = {}


def register(name: str, fn: Callable):
    """Register a host function of coordinates (``@register_symbolic`` in Symbolics).

    It must accept numpy arrays; it is evaluated on the host wherever it appears
    (for a nonlinear-Laplacian coefficient: at the interpolated half points).
    """
    _REGISTRY[name] = fn

    def call(*args):
        return Expr(("call", name) + tuple(_tree(a) for a in args))
    call.__name__ = name
    return call


class Equation:
    def __init__(self, lhs, rhs):
        self.lhs = _tree(lhs)
        self.rhs = _tree(rhs)

    def __repr__(self):
        return f"Equation({self.lhs!r} ~ {self.rhs!r})"


def Eq(lhs, rhs) -> Equation:
    """``lhs ~ rhs``."""
    return Equation(lhs, rhs)


class Interval:
    def __init__(self, lo: float, hi: float):
        self.lo = float(lo)
        self.hi = float(hi)


# ------------------------------------------------------------------------------------
# tree utilities
# ------------------------------------------------------------------------------------


def walk(t):
    yield t
    if isinstance(t, tuple) and t and isinstance(t[0], str):
        k = t[0]
        kids = []
        if k in ("add", "sub", "mul", "div", "pow"):
            kids = t[1:]
        elif k in ("neg",):
            kids = [t[1]]
        elif k == "fn":
            kids = [t[2]]
        elif k == "cmp":
            kids = [t[2], t[3]]
        elif k == "ifelse":
            kids = t[1:]
        elif k == "call":
            kids = t[2:]
        elif k == "D":
            kids = [t[3]]
        for c in kids:
            yield from walk(c)


def _linear_split(t, sign=1.0):
    """Additive terms of t as (sign, term)."""
    k = t[0]
    if k == "add":
        return _linear_split(t[1], sign) + _linear_split(t[2], sign) if len(t) == 3 else \
            [x for a in t[1:] for x in _linear_split(a, sign)]
    if k == "sub":
        return _linear_split(t[1], sign) + _linear_split(t[2], -sign)
    if k == "neg":
        return _linear_split(t[1], -sign)
    return [(sign, t)]


def _factors(t):
    k = t[0]
    if k == "mul":
        return [f for a in t[1:] for f in _factors(a)]
    return [t]


def _product(factors, sign):
    if not factors:
        out = ("num", 1.0)
    else:
        out = factors[0]
        for f in factors[1:]:
            out = ("mul", out, f)
    return ("neg", out) if sign < 0 else out


def _sum(terms):
    if not terms:
        return ("num", 0.0)
    out = terms[0]
    for t in terms[1:]:
        out = ("add", out, t)
    return out


class PDESystem:
    """``PDESystem(eqs, bcs, domains, ivs, dvs, ps)`` (ModelingToolkit)."""

    def __init__(self, eqs: Sequence[Equation], bcs: Sequence[Equation], domains, ivs: Sequence[IV],
                 dvs: Sequence[FieldApp], ps=(), name: str = "pdesys"):
        self.eqs = list(eqs) if isinstance(eqs, (list, tuple)) else [eqs]
        self.bcs = list(bcs)
        self.domains = {}
        for d in domains:
            iv, itv = d
            self.domains[iv.name] = (itv.lo, itv.hi) if isinstance(itv, Interval) else (float(itv[0]), float(itv[1]))
        self.ivs = [v.name for v in ivs]
        self.dvs = list(dvs)
        self.ps = list(ps)
        self.name = name

    def to_spec(self, disc) -> dict:
        tname = disc.time.name if disc.time is not None else None
        fields = [d.field.name for d in self.dvs]
        sig = {d.field.name: tuple(a.name for a in d.args) for d in self.dvs}
        spatial = [a for a in sig[fields[0]] if a != tname]
        for f in fields:
            if [a for a in sig[f] if a != tname] != spatial:
                raise NotImplementedError("all dependent variables must share the same spatial arguments")
        eqs = {}
        for e in self.eqs:
            lhs_terms = _linear_split(e.lhs)
            dt_terms = [(s, t) for s, t in lhs_terms if t[0] == "D" and t[1] == tname and t[2] == 1
                        and t[3][0] == "field"]
            if len(dt_terms) != 1 or dt_terms[0][0] != 1.0:
                raise NotImplementedError("each equation must contain one Dt(u) term with coefficient 1")
            f = dt_terms[0][1][3][1]
            rest = [("neg", t) if s > 0 else t for s, t in lhs_terms if (s, t) != dt_terms[0]]
            rhs = e.rhs
            for r in rest:
                rhs = ("add", rhs, r)
            eqs[f] = _strip_args(rhs)
        if sorted(eqs) != sorted(fields):
            raise ValueError("one equation per dependent variable is required")
        bcs, ics = [], {}
        for b in self.bcs:
            kind = _classify_bc(b, sig, tname, self.domains)
            if kind[0] == "ic":
                ics[kind[1]] = kind[2]
            else:
                bcs.append(kind[1])
        # one periodic entry per (field, iv)
        seen = set()
        uniq = []
        for b in bcs:
            key = (b["field"], b["iv"], b.get("side"), b["kind"])
            if b["kind"] == "periodic":
                key = (b["field"], b["iv"], None, "periodic")
            if key in seen:
                continue
            seen.add(key)
            uniq.append(b)
        if tname is not None:
            eqs = {k: _time_leaf(v, tname) for k, v in eqs.items()}
            for b in uniq:
                for key in ("a", "b", "g"):
                    if key in b:
                        b[key] = _time_leaf(b[key], tname)
        params = [(p.name, p.default) for p in self.ps]
        funcs = {}
        bc_trees = [b[k] for b in uniq for k in ("a", "b", "g") if isinstance(b.get(k), tuple)]
        for tree in list(eqs.values()) + list(ics.values()) + bc_trees:
            for n in walk(tree):
                if isinstance(n, tuple) and n and n[0] == "call":
                    funcs[n[1]] = _REGISTRY[n[1]]
        adv = disc.advection_scheme
        return {
            "time": tname,
            "ivs": spatial,
            "domain": dict(self.domains),
            "fields": fields,
            "params": params,
            "eqs": eqs,
            "bcs": uniq,
            "ics": ics,
            "functions": funcs,
            "disc": {"dxs": {k.name if isinstance(k, IV) else k: v for k, v in disc.dxs.items()},
                     "approx_order": disc.approx_order,
                     "advection": list(adv.spec()), "grid_align": disc.grid_align},
        }


def _time_leaf(t, tname):
    """The time variable appears as ('t',) in the spec."""
    if not isinstance(t, tuple) or not t:
        return t
    if t[0] == "iv":
        return ("t",) if t[1] == tname else t
    if t[0] in ("num", "param", "field", "t"):
        return t
    if t[0] == "D":
        return ("D", t[1], t[2], _time_leaf(t[3], tname))
    if t[0] == "fn":
        return ("fn", t[1], _time_leaf(t[2], tname))
    if t[0] == "cmp":
        return ("cmp", t[1], _time_leaf(t[2], tname), _time_leaf(t[3], tname))
    if t[0] == "call":
        return ("call", t[1]) + tuple(_time_leaf(a, tname) for a in t[2:])
    return (t[0],) + tuple(_time_leaf(a, tname) for a in t[1:])


def _strip_args(t):
    """Field applications carry their argument names; the spec uses ('field', name)."""
    if not isinstance(t, tuple):
        return t
    if t and t[0] == "field":
        return ("field", t[1])
    if t and t[0] in ("num", "param", "iv"):
        return t
    if t and t[0] == "fieldat":
        raise NotImplementedError("boundary-evaluated fields inside a PDE are not supported")
    if t and t[0] == "D":
        return ("D", t[1], t[2], _strip_args(t[3]))
    if t and t[0] == "fn":
        return ("fn", t[1], _strip_args(t[2]))
    if t and t[0] == "cmp":
        return ("cmp", t[1], _strip_args(t[2]), _strip_args(t[3]))
    if t and t[0] == "call":
        return ("call", t[1]) + tuple(_strip_args(a) for a in t[2:])
    return (t[0],) + tuple(_strip_args(a) for a in t[1:])


def _fieldat_info(t, sig, tname):
    """(field, {iv: value}) of a 'fieldat' node."""
    f = t[1]
    names = sig[f]
    vals = {}
    for k, v in enumerate(t[3]):
        if v is not None:
            vals[names[k]] = v
    return f, vals


def _classify_bc(b: Equation, sig, tname, domains):
    lhs, rhs = b.lhs, b.rhs
    # initial condition: u(x.., t0) ~ expr
    if lhs[0] == "fieldat":
        f, vals = _fieldat_info(lhs, sig, tname)
        if tname in vals and len(vals) == 1:
            return ("ic", f, _strip_args(rhs))
        if rhs[0] == "fieldat":
            f2, vals2 = _fieldat_info(rhs, sig, tname)
            (x, a), = vals.items()
            (x2, b2), = vals2.items()
            if f2 == f and x2 == x and {a, b2} == set(domains[x]):
                return ("bc", {"field": f, "iv": x, "kind": "periodic"})
            raise NotImplementedError("only periodic interface conditions u(x=a) ~ u(x=b) are supported")
    # robin family: a*u(x0) + b*Dx(u(x0)) ~ g
    terms = _linear_split(("sub", lhs, rhs))
    a_terms, b_terms, g_terms = [], [], []
    target = None
    for s, t in terms:
        fs = _factors(t)
        hit = None
        for i, fa in enumerate(fs):
            if fa[0] == "fieldat":
                hit = ("a", i, fa)
            elif fa[0] == "D" and fa[3][0] == "fieldat" and fa[2] == 1:
                hit = ("b", i, fa)
        if hit is None:
            g_terms.append(("neg", t) if s > 0 else t)
            continue
        kind, i, node = hit
        fnode = node if kind == "a" else node[3]
        f, vals = _fieldat_info(fnode, sig, tname)
        (x, xv), = vals.items()
        if kind == "b" and node[1] != x:
            raise NotImplementedError("boundary derivative must be normal to the boundary")
        key = (f, x, xv)
        if target is None:
            target = key
        elif target != key:
            raise NotImplementedError("a boundary condition may involve one field at one boundary")
        coef = _product(fs[:i] + fs[i + 1:], s)
        (a_terms if kind == "a" else b_terms).append(coef)
    if target is None:
        raise NotImplementedError(f"unrecognised boundary condition {b}")
    f, x, xv = target
    lo, hi = domains[x]
    side = "lo" if xv == lo else ("hi" if xv == hi else None)
    if side is None:
        raise NotImplementedError("boundary conditions must sit on the domain ends")
    return ("bc", {"field": f, "iv": x, "side": side, "kind": "robin",
                   "a": _strip_args(_sum(a_terms)), "b": _strip_args(_sum(b_terms)),
                   "g": _strip_args(_sum(g_terms))})
