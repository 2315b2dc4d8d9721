"""Lowering of a PDE system spec into the plain-data ``mol_problem_desc``.

This is the part of ``discretize`` that decides *what* the GPU computes; the
reference does the same work symbolically, point by point:

* grid construction (``src/discretization/discretize_vars.jl:219-285``),
* interior boxes (``src/system_parsing/interior_map.jl:1-10,53-139``),
* the DifferentialDiscretizer's tables (``differential_discretizer.jl:14-109``),
* rule classification (``generate_finite_difference_rules.jl:47-116``): nonlinear
  Laplacian, mixed derivatives, centered even orders, upwinded or WENO odd orders,
* boundary rows (``generate_bc_eqs.jl:35-58,238-328,396-459``).

Pointwise parts of the right-hand side become a register program.  Any
sub-expression that depends only on coordinates and constants is evaluated
once here (same IEEE operations, in the same order) and shipped as an aux
array: on GB300 an 8-byte load is far cheaper than a handful of FP64 ops.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from fractions import Fraction
from typing import Dict, List, Optional, Tuple

import numpy as np

from . import _lib as L
from .weights import (WENO_NU_ROW, Operator, centered, centered_nonuniform, extrapolator, half_centered,
                      half_centered_nonuniform, select, upwind, upwind_nonuniform, weno_nonuniform_rows, wrap)

# ------------------------------------------------------------------------------------
# grids (Julia Float64 ranges)
# ------------------------------------------------------------------------------------


def _rat(x: float):
    y = x
    a, d, b, c = 1, 1, 0, 0
    m = 2 ** 24
    while abs(y) <= m:
        f = int(y)
        y -= f
        a, c = f * a + c, a
        b, d = f * b + d, b
        if max(abs(a), abs(b)) > m:
            return c, d
        if b != 0 and a / b == x:
            break
        if y == 0:
            break
        y = 1.0 / y
    return a, b


def grid_points(lo: float, step: float, hi: float) -> np.ndarray:
    """Elements of ``lo:step:hi`` (rationalised when the inputs are exact ratios)."""
    sn, sd = _rat(step)
    if sd and sn / sd == step:
        an, ad = _rat(lo)
        on, od = _rat(hi)
        if ad and od and an / ad == lo and on / od == hi:
            den = ad * sd // math.gcd(ad, sd)
            a0, s0 = round(lo * den), round(step * den)
            n = max(0, (den * on - od * a0 + s0 * od) // (s0 * od))
            last = float(Fraction(a0 + (n - 1) * s0, den))
            nxt = float(Fraction(a0 + n * s0, den))
            if lo <= last <= hi + step / 2 and not (lo <= nxt <= hi):
                return np.array([float(Fraction(a0 + k * s0, den)) for k in range(n)])
    lf = (hi - lo) / step
    n = 0 if lf < 0 else (1 if lf == 0 else int(round(lf)) + 1)
    if lf > 0:
        stop2 = lo + (n - 1) * step
        n -= int(lo < hi < stop2) + int(lo > hi > stop2)
    flo, fst = Fraction(lo), Fraction(step)
    return np.array([float(flo + k * fst) for k in range(n)])


def make_axis(lo: float, hi: float, dxspec) -> Tuple[np.ndarray, float, bool]:
    """One dimension's grid (``discretize_space``, discretize_vars.jl:218-233): (points, step,
    uniform).

    An integer is a number of points and a float a step; the grid is then ``lo:dx:hi`` and
    its operators are the uniform tables.  When the step does not reach ``hi`` exactly the
    reference appends ``hi``; the grid is then a Vector, and so is a grid given as a
    sequence of points: every operator along it is built from the points themselves
    (differential_discretizer.jl:45-58, centered_diff_weights.jl:77-153)."""
    if isinstance(dxspec, (int, np.integer)) and not isinstance(dxspec, bool):
        dx = (hi - lo) / (int(dxspec) - 1)
    elif isinstance(dxspec, (float, np.floating)):
        dx = float(dxspec)
    else:
        g = np.array([float(v) for v in dxspec], dtype=np.float64)
        if g.ndim != 1 or len(g) < 2 or not np.all(np.diff(g) > 0):
            raise ValueError("a grid given as points must be strictly increasing, with at least two points")
        if g[-1] != hi:
            g = np.append(g, hi)
        return g, float(g[1] - g[0]), False
    g = grid_points(lo, dx, hi)
    if g[-1] != hi:
        return np.append(g, hi), dx, False
    return g, dx, True


def make_edge_axis(lo: float, hi: float, dxspec) -> Tuple[np.ndarray, float, bool]:
    """Edge-aligned grid (``generate_grid`` for EdgeAlignedGrid, discretize_vars.jl:373-390):
    the points ``(lo - dx/2):dx:(hi + dx/2)``, cell centres plus one ghost point beyond each
    end; an integer is a number of cells (``prepare_dx``, :284)."""
    if isinstance(dxspec, (int, np.integer)) and not isinstance(dxspec, bool):
        dx = (hi - lo) / int(dxspec)
    elif isinstance(dxspec, (float, np.floating)):
        dx = float(dxspec)
    else:
        raise NotImplementedError("edge-aligned grids given as points are not built")
    edges = grid_points(lo, dx, hi)
    if edges[-1] != hi:
        raise NotImplementedError("an edge-aligned grid whose step misses the end (a grid of midpoints) is not built")
    return grid_points(lo - dx / 2, dx, hi + dx / 2), dx, True


# ------------------------------------------------------------------------------------
# host evaluation of hoisted (coordinate-only) sub-expressions
# ------------------------------------------------------------------------------------

_NP_FN = {"sin": np.sin, "cos": np.cos, "tan": np.tan, "exp": np.exp, "log": np.log, "sqrt": np.sqrt,
          "abs": np.abs, "tanh": np.tanh, "sinh": np.sinh, "cosh": np.cosh, "atan": np.arctan}


def host_eval(t, coords: Dict[str, np.ndarray], functions, t_value=None):
    k = t[0]
    if k == "num":
        return t[1]
    if k == "iv":
        return coords[t[1]]
    if k == "t":
        return t_value
    if k in ("add", "mul"):
        acc = host_eval(t[1], coords, functions, t_value)
        for a in t[2:]:
            v = host_eval(a, coords, functions, t_value)
            acc = acc + v if k == "add" else acc * v
        return acc
    if k == "sub":
        return host_eval(t[1], coords, functions, t_value) - host_eval(t[2], coords, functions, t_value)
    if k == "div":
        return host_eval(t[1], coords, functions, t_value) / host_eval(t[2], coords, functions, t_value)
    if k == "neg":
        return -host_eval(t[1], coords, functions, t_value)
    if k == "pow":
        a = host_eval(t[1], coords, functions, t_value)
        if t[2][0] == "num" and float(t[2][1]).is_integer():
            n = int(t[2][1])
            if n == 2:
                return a * a
            if n == 3:
                return a * a * a
            if n == 1:
                return a
            if n == 0:
                return np.ones_like(a) if isinstance(a, np.ndarray) else 1.0
            if n == -1:
                return 1.0 / a
            if n == -2:
                return 1.0 / (a * a)
        return np.power(a, host_eval(t[2], coords, functions, t_value))
    if k == "fn":
        return _NP_FN[t[1]](host_eval(t[2], coords, functions, t_value))
    if k == "call":
        return functions[t[1]](*[host_eval(a, coords, functions, t_value) for a in t[2:]])
    if k == "cmp":
        a = host_eval(t[2], coords, functions, t_value)
        b = host_eval(t[3], coords, functions, t_value)
        r = {"<=": np.less_equal, "<": np.less, ">=": np.greater_equal, ">": np.greater, "==": np.equal}[t[1]](a, b)
        return np.asarray(r, dtype=np.float64) if isinstance(r, np.ndarray) else float(r)
    if k == "ifelse":
        c = host_eval(t[1], coords, functions, t_value)
        return np.where(np.asarray(c) != 0, host_eval(t[2], coords, functions, t_value),
                        host_eval(t[3], coords, functions, t_value))
    raise ValueError(f"cannot evaluate {k} on the host")


def eval_on_mesh(t, axes, ivs, functions, shape) -> np.ndarray:
    """host_eval of a coordinate-only expression at every point of the tensor grid `axes`
    (one 1-D coordinate array per dimension), as an array of `shape`.  Every operation is
    elementwise, so the grid is cut into slabs of its last dimension evaluated on a thread
    pool (numpy releases the GIL inside its loops): the values are those of one evaluation
    over the whole mesh, and a 256^3 face array takes seconds instead of a minute."""
    import os
    from concurrent.futures import ThreadPoolExecutor
    total = int(np.prod(shape))
    nlast = len(axes[-1]) if axes else 1
    workers = max(1, min(os.cpu_count() or 1, 32, nlast))
    if total < (1 << 18) or workers == 1 or len(axes) == 0:
        mesh = np.meshgrid(*axes, indexing="ij")
        v = host_eval(t, {x: g for x, g in zip(ivs, mesh)}, functions)
        return np.broadcast_to(np.asarray(v, dtype=np.float64), shape).copy()
    out = np.empty(shape, dtype=np.float64)
    bounds = np.linspace(0, nlast, min(nlast, 4 * workers) + 1).astype(int)

    def slab(k):
        a, b = int(bounds[k]), int(bounds[k + 1])
        if b <= a:
            return
        sub = list(axes[:-1]) + [axes[-1][a:b]]
        mesh = np.meshgrid(*sub, indexing="ij")
        v = host_eval(t, {x: g for x, g in zip(ivs, mesh)}, functions)
        out[..., a:b] = np.broadcast_to(np.asarray(v, dtype=np.float64), shape[:-1] + (b - a,))

    with ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(slab, range(len(bounds) - 1)))
    return out


def _leaves(t):
    """Set of leaf kinds in t ('field', 'param', 'iv', 't', 'D', 'term', ...)."""
    k = t[0]
    if k in ("num", "param", "iv", "t", "field", "term", "faceaux", "aux"):
        return {k}
    if k == "D":
        return {"D"}
    if k == "upwind":
        return {"term"}
    out = set()
    kids = t[2:] if k in ("fn", "call") else (t[2:] if k == "cmp" else t[1:])
    for a in kids:
        if isinstance(a, tuple):
            out |= _leaves(a)
    return out


# ------------------------------------------------------------------------------------
# register-machine compiler
# ------------------------------------------------------------------------------------


class ProgramBuilder:
    """Compiles expression trees to straight-line register code with CSE and register reuse."""

    def __init__(self, lowered: "Lowered", kind: str, max_regs: int):
        self.lw = lowered
        self.kind = kind          # "cell" | "face" | "bc"
        self.max_regs = max_regs
        self.instrs: List[Tuple[int, int, int, int, int, int]] = []  # op, dst, a, b, c, imm (virtual regs)
        self.memo: Dict[tuple, int] = {}
        self.nv = 0

    def _new(self):
        self.nv += 1
        return self.nv - 1

    def emit(self, op, a=0, b=0, c=0, imm=0):
        v = self._new()
        self.instrs.append((op, v, a, b, c, imm))
        return v

    def value(self, t) -> int:
        if t in self.memo:
            return self.memo[t]
        k = t[0]
        lw = self.lw
        if k == "num":
            v = self.emit(L.OP_CONST, imm=lw.const(t[1]))
        elif k == "param":
            v = self.emit(L.OP_PARAM, imm=lw.param_index(t[1]))
        elif k == "field":
            v = self.emit(L.OP_FIELD, imm=lw.fields.index(t[1]))
        elif k == "aux":
            v = self.emit(L.OP_AUX, imm=t[1])
        elif k == "faceaux":
            v = self.emit(L.OP_AUX, imm=t[1])
        elif k == "iv":
            v = self.emit(L.OP_COORD, imm=lw.ivs.index(t[1]))
        elif k == "t":
            v = self.emit(L.OP_TIME)
        elif k == "term":
            v = self.emit(L.OP_TERM, imm=t[1])
        elif k == "upwind":
            kap = self.value(t[1])
            v = self.emit(L.OP_UPWIND, a=kap, b=t[2], c=t[3])
        elif k in ("add", "mul"):
            op = L.OP_ADD if k == "add" else L.OP_MUL
            v = self.value(t[1])
            for a in t[2:]:
                w = self.value(a)
                v = self.emit(op, a=v, b=w)
        elif k in ("sub", "div"):
            a = self.value(t[1])
            b = self.value(t[2])
            v = self.emit(L.OP_SUB if k == "sub" else L.OP_DIV, a=a, b=b)
        elif k == "neg":
            v = self.emit(L.OP_NEG, a=self.value(t[1]))
        elif k == "pow":
            if t[2][0] == "num" and float(t[2][1]).is_integer() and abs(t[2][1]) <= 64:
                v = self.emit(L.OP_POWI, a=self.value(t[1]), imm=int(t[2][1]))
            else:
                v = self.emit(L.OP_POW, a=self.value(t[1]), b=self.value(t[2]))
        elif k == "fn":
            v = self.emit(L.OP_FN, a=self.value(t[2]), imm=L.FN_IDS[t[1]])
        elif k == "cmp":
            v = self.emit(L.OP_CMP, a=self.value(t[2]), b=self.value(t[3]), imm=L.CMP_IDS[t[1]])
        elif k == "ifelse":
            v = self.emit(L.OP_IFELSE, a=self.value(t[1]), b=self.value(t[2]), c=self.value(t[3]))
        else:
            raise NotImplementedError(f"cannot compile node {k}")
        self.memo[t] = v
        return v

    def out(self, t, index: int):
        v = self.value(t)
        self.instrs.append((L.OP_OUT, 0, v, 0, 0, index))

    _READS = {}

    @staticmethod
    def _reg_slots(op):
        """Operand slots (1=a, 2=b, 3=c) that hold registers for opcode `op`."""
        if op in (L.OP_NEG, L.OP_POWI, L.OP_FN, L.OP_OUT, L.OP_UPWIND):
            return (2,)
        if op in (L.OP_ADD, L.OP_SUB, L.OP_MUL, L.OP_DIV, L.OP_POW, L.OP_CMP):
            return (2, 3)
        if op == L.OP_IFELSE:
            return (2, 3, 4)
        return ()

    def finish(self) -> List[Tuple[int, int, int, int, int, int]]:
        """Map virtual registers to at most max_regs physical registers (linear scan).

        A destination may reuse a register read by the same instruction: the device reads
        every operand before it writes the result.
        """
        last = {}
        for pc, ins in enumerate(self.instrs):
            for s in self._reg_slots(ins[0]):
                last[ins[s]] = pc
        free = list(range(self.max_regs))[::-1]
        phys = {}
        out = []
        for pc, ins in enumerate(self.instrs):
            op = ins[0]
            row = list(ins)
            slots = self._reg_slots(op)
            for s in slots:
                row[s] = phys[ins[s]]
            for s in slots:
                v = ins[s]
                if last.get(v) == pc and v in phys:
                    free.append(phys.pop(v))
            if op != L.OP_OUT:
                if not free:
                    raise NotImplementedError(f"program needs more than {self.max_regs} registers")
                pd = free.pop()
                if ins[1] in last:
                    phys[ins[1]] = pd
                else:
                    free.append(pd)
                row[1] = pd
            else:
                row[1] = 0
            out.append(tuple(row))
        return out


# ------------------------------------------------------------------------------------
# lowering
# ------------------------------------------------------------------------------------


@dataclass
class Lowered:
    ivs: List[str]
    fields: List[str]
    param_names: List[str]
    param_values: np.ndarray
    grids: List[np.ndarray]
    dx: List[float]
    npts: List[int]
    lower: List[int]
    upper: List[int]
    periodic: Dict[str, List[bool]]
    functions: dict
    order: int
    adv: list
    ops: List[Operator] = field(default_factory=list)
    op_keys: Dict[tuple, int] = field(default_factory=dict)
    terms: List[dict] = field(default_factory=list)
    term_keys: Dict[tuple, int] = field(default_factory=dict)
    consts: List[float] = field(default_factory=list)
    const_keys: Dict[float, int] = field(default_factory=dict)
    aux: List[np.ndarray] = field(default_factory=list)
    aux_keys: Dict[tuple, int] = field(default_factory=dict)
    programs: List[List[tuple]] = field(default_factory=list)
    cell_prog: int = -1
    bcs: Dict[tuple, dict] = field(default_factory=dict)
    u0: Optional[np.ndarray] = None
    spec: Optional[dict] = None
    uniform: List[bool] = field(default_factory=list)

    # -- registries
    def const(self, v: float) -> int:
        key = float(v)
        k = (key, math.copysign(1.0, key))
        if k not in self.const_keys:
            self.const_keys[k] = len(self.consts)
            self.consts.append(key)
        return self.const_keys[k]

    def param_index(self, name: str) -> int:
        return self.param_names.index(name)

    def op(self, kind: str, j: int, d: int, p: int = 0) -> int:
        key = (kind, j, d, p)
        if key not in self.op_keys:
            dx = self.dx[j]
            if kind == "weno_nu":            # per-point WENO geometry (nonuniform_weno.jl)
                rows = weno_nonuniform_rows(self.grids[j])
                o = Operator(WENO_NU_ROW, 0, rows[0], [], [], 0, 0, 0, rows)
            elif self.uniform and not self.uniform[j]:
                if kind == "centered":
                    o = centered_nonuniform(d, self.order, self.grids[j])
                elif kind in ("half", "interp", "half_outer"):
                    g = self.grids[j]
                    if kind == "half_outer":
                        # differential_discretizer.jl:47-52: the nonlinear Laplacian's outer
                        # operator is built on the grid's midpoints
                        o = half_centered_nonuniform(d, self.order, [(g[i + 1] + g[i]) / 2 for i in range(len(g) - 1)])
                    elif kind == "half":
                        o = half_centered_nonuniform(d, self.order, g)
                    else:
                        o = half_centered_nonuniform(0, max(4, self.order), g)
                elif kind in ("wind_pos", "wind_neg") and d + p == 2:
                    # the reference's nonuniform tables reach every interior point only for L = 2
                    o = upwind_nonuniform(d, p, self.grids[j], d + p - 1 if kind == "wind_pos" else 0)
                else:
                    raise NotImplementedError(
                        f"{kind} operators (order {d}, upwind order {p}) on the nonuniform grid of {self.ivs[j]} "
                        "are not built (centered derivatives, first-order upwinding, the nonlinear Laplacian "
                        "and boundary rows are)")
            elif kind == "centered":
                o = centered(d, self.order, dx)
            elif kind == "wind_pos":       # offside d+p-1: backward taps (windmap[2])
                o = upwind(d, p, dx, d + p - 1)
            elif kind == "wind_neg":       # offside 0: forward taps (windmap[1])
                o = upwind(d, p, dx, 0)
            elif kind == "half":
                o = half_centered(d, self.order, dx)
            elif kind == "interp":
                o = half_centered(0, max(4, self.order), dx)
            elif kind == "extrap":          # BoundaryInterpolatorExtrapolator(max(6, order), dx)
                o = extrapolator(max(6, self.order))
            else:
                raise ValueError(kind)
            self.op_keys[key] = len(self.ops)
            self.ops.append(o)
        return self.op_keys[key]

    def term(self, **kw) -> int:
        key = tuple(sorted((k, v if not isinstance(v, list) else tuple(v)) for k, v in kw.items()))
        if key not in self.term_keys:
            self.term_keys[key] = len(self.terms)
            self.terms.append(kw)
        return self.term_keys[key]

    @property
    def ncell(self) -> int:
        return int(np.prod([self.npts[j] - self.lower[j] - self.upper[j] for j in range(len(self.ivs))]))

    @property
    def interior_shape(self):
        return tuple(self.npts[j] - self.lower[j] - self.upper[j] for j in range(len(self.ivs)))

    @property
    def n_unknowns(self) -> int:
        return self.ncell * len(self.fields)

    def interior_coords(self) -> Dict[str, np.ndarray]:
        axes = [self.grids[j][self.lower[j]:self.npts[j] - self.upper[j]] for j in range(len(self.ivs))]
        mesh = np.meshgrid(*axes, indexing="ij")
        return {self.ivs[j]: mesh[j] for j in range(len(self.ivs))}


def _split_add(t, sign=1.0):
    k = t[0]
    if k == "add":
        return [x for a in t[1:] for x in _split_add(a, sign)]
    if k == "sub":
        return _split_add(t[1], sign) + _split_add(t[2], -sign)
    if k == "neg":
        return _split_add(t[1], -sign)
    return [(sign, t)]


def _deriv_orders(t, x) -> set:
    """Orders of the derivatives along x anywhere in the expression (``d_orders``)."""
    out = set()
    if isinstance(t, tuple) and t:
        if t[0] == "D" and t[1] == x:
            out.add(t[2])
        for a in t[1:]:
            if isinstance(a, tuple):
                out |= _deriv_orders(a, x)
    return out


def _subst_iv(t, x, val):
    if not isinstance(t, tuple) or not t:
        return t
    if t[0] == "iv" and t[1] == x:
        return val
    return tuple(_subst_iv(a, x, val) if isinstance(a, tuple) else a for a in t)


def _is_zero(t) -> bool:
    return _leaves(t) <= {"num"} and float(host_eval(t, {}, {})) == 0.0


def _split_mul(t):
    k = t[0]
    if k == "mul":
        num, den = [], []
        for a in t[1:]:
            n2, d2 = _split_mul(a)
            num += n2
            den += d2
        return num, den
    if k == "div":
        n1, d1 = _split_mul(t[1])
        n2, d2 = _split_mul(t[2])
        return n1 + d2, d1 + n2
    if k == "neg":
        n1, d1 = _split_mul(t[1])
        return [("num", -1.0)] + n1, d1
    return [t], []


def _fold(op, items):
    out = items[0]
    for a in items[1:]:
        out = (op, out, a)
    return out


class _Lowerer:
    def __init__(self, spec: dict):
        self.spec = spec
        ivs = list(spec["ivs"])
        if not 1 <= len(ivs) <= 3:
            raise NotImplementedError("1 to 3 spatial dimensions are supported")
        fields = list(spec["fields"])
        disc = spec["disc"]
        align = disc.get("grid_align", "center")
        if align not in ("center", "edge"):
            raise NotImplementedError(f"grid alignment {align!r} is not built (center and edge are)")
        self.edge = align == "edge"
        grids, dxs, uniform = [], [], []
        for x in ivs:
            lo, hi = spec["domain"][x]
            if self.edge:
                g, dx, uni = make_edge_axis(float(lo), float(hi), disc["dxs"][x])
            else:
                g, dx, uni = make_axis(float(lo), float(hi), disc["dxs"][x])
            grids.append(g)
            dxs.append(dx)
            uniform.append(uni)
        npts = [len(g) for g in grids]
        periodic = {f: [False] * len(ivs) for f in fields}
        bcs = {}
        for b in spec.get("bcs", []):
            j = ivs.index(b["iv"])
            if b["kind"] == "periodic":
                periodic[b["field"]][j] = True
            else:
                bcs[(b["field"], j, b["side"])] = b
        adv = list(disc.get("advection", ["upwind", 1]))
        lower = None
        upper = None
        self.extrap_dims = set()
        for f in fields:
            lo_ = [1 if periodic[f][j] else int((f, j, "lo") in bcs) for j in range(len(ivs))]
            up_ = [0 if periodic[f][j] else int((f, j, "hi") in bcs) for j in range(len(ivs))]
            if adv[0] == "weno":
                # stencil extents (interior_map.jl:83-90, :117-139): WENO along a bounded uniform
                # dimension reaches 2 (WENO.jl:94), so the interior of an equation with a first
                # derivative along it stops two points from each end and point 2 (n-1) is
                # extrapolated (generate_extrap_eqs!, generate_bc_eqs.jl:336-392)
                for j, x in enumerate(ivs):
                    if periodic[f][j] or 1 not in _deriv_orders(spec["eqs"][f], x):
                        continue
                    if self.edge:
                        raise NotImplementedError("WENO along a bounded edge-aligned dimension is not built")
                    if not uniform[j]:
                        continue        # extent 0 on a nonuniform grid (WENO.jl:95): no extrapolation
                    for side, arr in (("lo", lo_), ("hi", up_)):
                        b = bcs.get((f, j, side))
                        if b is None:
                            raise NotImplementedError(
                                f"WENO along {x} with no boundary row at one end (two coupled extrapolated points) "
                                "is not built")
                        if not _is_zero(b["b"]):
                            raise NotImplementedError(
                                f"WENO along {x} next to a Neumann/Robin row (a coupled boundary/extrapolation "
                                "pair) is not built")
                        arr[j] = max(arr[j], 2)
                    self.extrap_dims.add((f, j))
            if lower is None:
                lower, upper = lo_, up_
            elif lo_ != lower or up_ != upper:
                raise NotImplementedError("all fields must share one interior box")
        params = spec.get("params", [])
        self.lw = Lowered(ivs=ivs, fields=fields, param_names=[p[0] for p in params],
                          param_values=np.array([float(p[1]) for p in params], dtype=np.float64),
                          grids=grids, dx=dxs, npts=npts, lower=lower, upper=upper, periodic=periodic,
                          functions=dict(spec.get("functions", {})), order=int(disc.get("approx_order", 2)),
                          adv=adv, spec=spec, uniform=uniform)
        for j in range(len(ivs)):
            if self.edge and any(periodic[f][j] for f in fields):
                raise NotImplementedError("periodic boundaries on an edge-aligned grid are not built")
            if not uniform[j] and any(periodic[f][j] for f in fields):
                # centered_difference.jl:36 asserts that no interface boundary meets a nonuniform dimension
                raise NotImplementedError(f"periodic boundaries on the nonuniform grid of {ivs[j]}")
        self.bcs = bcs
        if self.lw.order % 2:
            # MOLFiniteDifference warns and keeps the odd order (MOLFiniteDifference.jl:56-58)
            pass

    # ---------------------------------------------------------------- derivative terms
    def deriv_term(self, node, field_ctx=None) -> int:
        _, x, d, arg = node
        lw = self.lw
        j = lw.ivs.index(x)
        if arg[0] == "field":
            f = lw.fields.index(arg[1])
            if d % 2 == 0:
                return lw.term(kind=L.TERM_LINEAR, field=f, dim=j, op=lw.op("centered", j, d))
            if lw.adv[0] == "weno" and d == 1:
                if not lw.uniform[j]:
                    # node-centred Lagrange WENO-5 from the grid's coordinates (nonuniform_weno.jl)
                    return lw.term(kind=L.TERM_WENO, field=f, dim=j, eps=float(lw.adv[1]), dx=1.0,
                                   op=lw.op("weno_nu", j, 0), variant=1)
                return lw.term(kind=L.TERM_WENO, field=f, dim=j, eps=float(lw.adv[1]), dx=lw.dx[j])
            # bare odd derivative: positive wind (upwind_difference.jl:278-302)
            p = int(lw.adv[1]) if lw.adv[0] == "upwind" else 1
            return lw.term(kind=L.TERM_LINEAR, field=f, dim=j, op=lw.op("wind_pos", j, d, p))
        if arg[0] == "D" and d == 1 and arg[2] == 1 and arg[3][0] == "field":
            k = lw.ivs.index(arg[1])
            f = lw.fields.index(arg[3][1])
            return lw.term(kind=L.TERM_MIXED, field=f, dim=j, dim2=k, op=lw.op("centered", j, 1),
                           op2=lw.op("centered", k, 1))
        if d == 1:
            num, den = _split_mul(arg)
            ks = [i for i, a in enumerate(num) if a[0] == "D" and a[1] == x and a[2] == 1 and a[3][0] == "field"]
            if ks:
                inner = num[ks[0]]
                coef_num = num[:ks[0]] + num[ks[0] + 1:]
                return self.nonlinlap_term(coef_num, den, inner[3][1], j)
        raise NotImplementedError(f"unsupported derivative form {node}")

    def nonlinlap_term(self, coef_num, coef_den, g, j) -> int:
        lw = self.lw
        f = lw.fields.index(g)
        # coefficient a(x, u, p) at the half point, built like the oracle/reference: product then quotients
        a = None
        for c in coef_num:
            a = c if a is None else ("mul", a, c)
        for c in coef_den:
            a = ("div", ("num", 1.0), c) if a is None else ("div", a, c)
        prog = -1
        aux0 = -1
        if a is not None:
            a, faux = self.hoist_face(a, j, f)
            pb = ProgramBuilder(lw, "face", L.MOL_MAX_REGS)
            pb.out(a, 0)
            lw.programs.append(pb.finish())
            prog = len(lw.programs) - 1
            aux0 = faux[0] if faux else 0
        outer = lw.op("half" if (not lw.uniform or lw.uniform[j]) else "half_outer", j, 1)
        return lw.term(kind=L.TERM_NONLINLAP, field=f, dim=j, op=outer, op2=lw.op("half", j, 1),
                       op3=lw.op("interp", j, 0), prog=prog, aux0=aux0, key=repr(a))

    # ---------------------------------------------------------------- hoisting
    def _hoistable(self, t) -> bool:
        lv = _leaves(t)
        return lv <= {"num", "iv"} and "iv" in lv

    def hoist_cell(self, t):
        """Replace coordinate-only sub-expressions by cell aux arrays; fold constants."""
        if not isinstance(t, tuple):
            return t
        k = t[0]
        if k in ("num", "param", "field", "t", "term"):
            return t
        if k == "iv":
            return t
        if self._hoistable(t):
            return self._cell_aux(t)
        if k == "upwind":
            return ("upwind", self.hoist_cell(t[1]), t[2], t[3])
        if k in ("fn",):
            return (k, t[1], self.hoist_cell(t[2]))
        if k == "cmp":
            return (k, t[1], self.hoist_cell(t[2]), self.hoist_cell(t[3]))
        if k == "call":
            raise NotImplementedError("registered functions of the state are not supported")
        return (k,) + tuple(self.hoist_cell(a) for a in t[1:])

    def _cell_aux(self, t):
        lw = self.lw
        key = ("cell", t)
        if key not in lw.aux_keys:
            axes = [lw.grids[j][lw.lower[j]:lw.npts[j] - lw.upper[j]] for j in range(len(lw.ivs))]
            arr = eval_on_mesh(t, axes, lw.ivs, lw.functions, tuple(lw.interior_shape))
            lw.aux_keys[key] = len(lw.aux)
            lw.aux.append(np.ascontiguousarray(arr.reshape(-1, order="F")))
        return ("aux", lw.aux_keys[key])

    def _hoist_bc_calls(self, t, j, side):
        """Registered functions of coordinates in a boundary row (docs: boundary_conditions.md,
        "Registered User Defined Function") are evaluated on the host at every point of the
        boundary face (its own coordinate fixed at the domain's end, the others the grid's)
        into a full-grid array the row's program reads at its boundary point."""
        if not isinstance(t, tuple) or not t:
            return t
        if t[0] == "call" and _leaves(t) <= {"num", "iv"}:
            lw = self.lw
            key = ("bc", j, side, t)
            if key not in lw.aux_keys:
                grids = np.meshgrid(*lw.grids, indexing="ij")
                coords = {x: g for x, g in zip(lw.ivs, grids)}
                v = host_eval(t, coords, lw.functions)
                arr = np.broadcast_to(np.asarray(v, dtype=np.float64), tuple(lw.npts))
                lw.aux_keys[key] = len(lw.aux)
                lw.aux.append(np.ascontiguousarray(arr.reshape(-1, order="F")))
            return ("aux", lw.aux_keys[key])
        if t[0] in ("fn", "call"):
            return t[:2] + tuple(self._hoist_bc_calls(a, j, side) for a in t[2:])
        if t[0] == "cmp":
            return t[:2] + tuple(self._hoist_bc_calls(a, j, side) for a in t[2:])
        return (t[0],) + tuple(self._hoist_bc_calls(a, j, side) if isinstance(a, tuple) else a for a in t[1:])

    def hoist_face(self, t, j, f):
        """Hoist coordinate-only parts of a nonlinear-Laplacian coefficient into face arrays.

        The coordinate along j at half point I+1/2 is the interpolated one the reference uses,
        dot(interp weights, grid[wrapped taps]) (nonlinear_laplacian.jl:74-83); the other
        coordinates are the cell's.
        """
        lw = self.lw
        faux: List[int] = []
        memo: Dict[tuple, int] = {}

        def rec(t):
            if not isinstance(t, tuple):
                return t
            k = t[0]
            if k in ("num", "param", "field", "t"):
                return t
            if k == "iv" or self._hoistable(t):
                if t not in memo:
                    memo[t] = self._face_aux(t, j, f)
                    faux.append(memo[t])
                return ("faceaux", memo[t])
            if k == "fn":
                return (k, t[1], rec(t[2]))
            if k == "cmp":
                return (k, t[1], rec(t[2]), rec(t[3]))
            if k == "call":
                raise NotImplementedError("registered functions of the state are not supported")
            return (k,) + tuple(rec(a) for a in t[1:])

        out = rec(t)
        # face-aux indices are relative to the term's first aux array; they are allocated
        # contiguously so aux0 + k addresses the k-th one
        if faux:
            base = faux[0]
            out = _rebase_faceaux(out, base)
        return out, faux

    def _face_aux(self, t, j, f):
        lw = self.lw
        n = lw.npts[j]
        per = lw.periodic[lw.fields[f]][j]
        interp = lw.ops[lw.op("interp", j, 0)]
        nd = len(lw.ivs)
        ext = [lw.npts[k] + (1 if k == j else 0) for k in range(nd)]
        # interpolated coordinate at each half point index Ih (0..n)
        xh = np.zeros(n + 1)
        valid = np.zeros(n + 1, dtype=bool)
        for Ih in range(1, n + 1 if per else n):
            w, taps = select(interp, Ih, n, per)
            if per:
                taps = [wrap(q, n) for q in taps]
            acc = None
            for wk, tk in zip(w, taps):
                term = wk * lw.grids[j][tk - 1]
                acc = term if acc is None else acc + term
            xh[Ih] = acc
            valid[Ih] = True
        axes = []
        for k in range(nd):
            if k == j:
                axes.append(xh)
            else:
                axes.append(lw.grids[k])
        v = eval_on_mesh(t, axes, lw.ivs, lw.functions, tuple(ext))
        sl = [slice(None)] * nd
        sl[j] = ~valid
        v[tuple(sl)] = 0.0
        idx = len(lw.aux)
        lw.aux.append(np.ascontiguousarray(v.reshape(-1, order="F")))
        return idx

    # ---------------------------------------------------------------- right-hand side
    def rhs_tree(self, f: str):
        """The field's RHS with derivatives replaced by term references (and upwind selects)."""
        lw = self.lw
        out = []
        for sign, term in _split_add(self.spec["eqs"][f]):
            num, den = _split_mul(term)
            sph = self.spherical_tree(num, den)
            if sph is not None:
                out.append(("neg", sph) if sign < 0 else sph)
                continue
            odd = [k for k, a in enumerate(num) if a[0] == "D" and a[3][0] == "field" and a[2] % 2 == 1
                   and not (lw.adv[0] == "weno" and a[2] == 1)]
            if odd:
                kd = odd[0]
                dn = num[kd]
                j = lw.ivs.index(dn[1])
                fi = lw.fields.index(dn[3][1])
                p = int(lw.adv[1]) if lw.adv[0] == "upwind" else 1
                tpos = lw.term(kind=L.TERM_LINEAR, field=fi, dim=j, op=lw.op("wind_pos", j, dn[2], p))
                tneg = lw.term(kind=L.TERM_LINEAR, field=fi, dim=j, op=lw.op("wind_neg", j, dn[2], p))
                others = [self.subst(a) for a in num[:kd] + num[kd + 1:]]
                kap = None
                for a in others:
                    kap = a if kap is None else ("mul", kap, a)
                for dd in den:
                    dv = self.subst(dd)
                    kap = ("div", ("num", 1.0), dv) if kap is None else ("div", kap, dv)
                if kap is None:
                    kap = ("num", 1.0)
                if sign < 0:
                    kap = ("neg", kap)
                out.append(("upwind", kap, tpos, tneg))
            else:
                v = self.subst(term)
                out.append(("neg", v) if sign < 0 else v)
        return _fold("add", out)

    def spherical_tree(self, num, den):
        """The spherical Laplacian ``r^-2 Dr(c r^2 Dr(u))`` (generate_spherical_diffusion_rules,
        spherical_laplacian.jl:42-130): a product whose only denominator is r^2 and which has a
        factor Dr(inner), inner a product of r^2, Dr(u) and coefficient factors c, becomes the
        other factors times spherical_diffusion(c) (:10-40), which the reference writes as
        c(cell) * (D1(u) / r + Dr(c Dr(u))): the centered first derivative over the cell's r
        plus the nonlinear Laplacian of c.  None when the term does not have that form."""
        lw = self.lw
        for kd, a in enumerate(num):
            if a[0] != "D" or a[2] != 1 or a[3][0] == "field":
                continue
            x = a[1]
            r2 = ("pow", ("iv", x), ("num", 2.0))
            inum, iden = _split_mul(a[3])
            if den != [r2] or iden or inum.count(r2) != 1:
                continue
            dk = [k for k, q in enumerate(inum) if q[0] == "D" and q[1] == x and q[2] == 1 and q[3][0] == "field"]
            if len(dk) != 1:
                continue
            g = lw.fields.index(inum[dk[0]][3][1])
            coef = [q for k, q in enumerate(inum) if k != dk[0] and q != r2]
            j = lw.ivs.index(x)
            if np.any(np.abs(lw.grids[j][lw.lower[j]:lw.npts[j] - lw.upper[j]]) <= 1e-6):
                # spherical_laplacian.jl:30-33: 6 c D2(u) at r = 0
                raise NotImplementedError("a spherical Laplacian with r = 0 as an unknown is not built")
            here = _fold("mul", [self.subst(c) for c in coef]) if coef else ("num", 1.0)
            d1 = lw.term(kind=L.TERM_LINEAR, field=g, dim=j, op=lw.op("centered", j, 1))
            nll = self.nonlinlap_term(coef, [], lw.fields[g], j)
            v = ("mul", here, ("add", ("div", ("term", d1), ("iv", x)), ("term", nll)))
            for k, q in enumerate(num):
                if k != kd:
                    v = ("mul", self.subst(q), v)
            return v
        return None

    def subst(self, t):
        k = t[0]
        if k == "D":
            return ("term", self.deriv_term(t))
        if k in ("num", "param", "field", "iv", "t"):
            return t
        if k == "fn":
            return (k, t[1], self.subst(t[2]))
        if k == "cmp":
            return (k, t[1], self.subst(t[2]), self.subst(t[3]))
        if k == "call":
            return (k, t[1]) + tuple(self.subst(a) for a in t[2:])
        return (k,) + tuple(self.subst(a) for a in t[1:])

    def build(self) -> Lowered:
        lw = self.lw
        pb = ProgramBuilder(lw, "cell", L.MOL_MAX_REGS)
        trees = []
        for f in lw.fields:
            trees.append(self.hoist_cell(self.rhs_tree(f)))
        for i, t in enumerate(trees):
            pb.out(t, i)
        lw.programs.append(pb.finish())
        lw.cell_prog = len(lw.programs) - 1
        # boundary rows
        for (f, j, side), b in self.bcs.items():
            # the row's own coordinate is the domain's end (axiesvals, discretize_vars.jl:321-330)
            xe = ("num", float(self.spec["domain"][lw.ivs[j]][0 if side == "lo" else 1]))
            a, bb, g = (self._hoist_bc_calls(_subst_iv(b[k], lw.ivs[j], xe), j, side) for k in ("a", "b", "g"))
            if self.edge:
                # the face half-way between the ghost point and the first (last) unknown:
                # a * interpolation + b * half-offset derivative (generate_bc_eqs.jl:80-160)
                entry = {"kind": L.BC_EDGE, "op": lw.op("half", j, 1), "iop": lw.op("interp", j, 0), "prog": -1,
                         "a": 0.0, "b": 0.0, "g": 0.0, "extrap": 0}
            else:
                entry = {"kind": L.BC_ROBIN, "op": lw.op("centered", j, 1), "prog": -1, "a": 0.0, "b": 0.0,
                         "g": 0.0, "extrap": 1 + lw.op("extrap", j, 0) if (f, j) in self.extrap_dims else 0}
            lv = _leaves(a) | _leaves(bb) | _leaves(g)
            if lv <= {"num"}:
                entry["a"] = float(host_eval(a, {}, {}))
                entry["b"] = float(host_eval(bb, {}, {}))
                entry["g"] = float(host_eval(g, {}, {}))
            else:
                if lv & {"field", "D", "call"}:
                    raise NotImplementedError("boundary conditions may depend on t, x and parameters only")
                bp = ProgramBuilder(lw, "bc", 16)
                bp.out(a, 0)
                bp.out(bb, 1)
                bp.out(g, 2)
                lw.programs.append(bp.finish())
                entry["prog"] = len(lw.programs) - 1
            lw.bcs[(lw.fields.index(f), j, 0 if side == "lo" else 1)] = entry
        for f in lw.fields:
            for j in range(len(lw.ivs)):
                if lw.periodic[f][j]:
                    lw.bcs[(lw.fields.index(f), j, 0)] = {"kind": L.BC_PERIODIC, "op": 0, "prog": -1,
                                                          "a": 0.0, "b": 0.0, "g": 0.0}
        # initial condition at the interior points (generate_ic_defaults.jl:1-27)
        ics = self.spec.get("ics", {})
        if all(f in ics for f in lw.fields):
            coords = lw.interior_coords()
            t0 = float(self.spec["domain"][self.spec["time"]][0]) if self.spec.get("time") in self.spec["domain"] else 0.0
            parts = []
            for f in lw.fields:
                v = host_eval(ics[f], coords, lw.functions, t0)
                parts.append(np.broadcast_to(np.asarray(v, dtype=np.float64), lw.interior_shape).reshape(-1, order="F"))
            lw.u0 = np.ascontiguousarray(np.concatenate(parts))
        return lw


def _rebase_faceaux(t, base):
    if not isinstance(t, tuple):
        return t
    if t[0] == "faceaux":
        return ("faceaux", t[1] - base)
    if t[0] in ("num", "param", "field", "t", "iv"):
        return t
    if t[0] in ("fn",):
        return (t[0], t[1], _rebase_faceaux(t[2], base))
    if t[0] == "cmp":
        return (t[0], t[1], _rebase_faceaux(t[2], base), _rebase_faceaux(t[3], base))
    return (t[0],) + tuple(_rebase_faceaux(a, base) for a in t[1:])


def lower(spec: dict) -> Lowered:
    return _Lowerer(spec).build()


# ------------------------------------------------------------------------------------
# ctypes descriptor
# ------------------------------------------------------------------------------------


class Descriptor:
    """A filled ``mol_problem_desc`` plus the host arrays it points to (kept alive here)."""

    def __init__(self, lw: Lowered):
        self.lw = lw
        keep = []
        d = L.mol_problem_desc()
        d.abi_version = L.MOL_ABI_VERSION
        nd = len(lw.ivs)
        d.ndim = nd
        d.nfields = len(lw.fields)
        d.nparams = len(lw.param_names)
        for j in range(nd):
            d.npts[j] = lw.npts[j]
            d.lower[j] = lw.lower[j]
            d.upper[j] = lw.upper[j]
            d.dx[j] = lw.dx[j]
            g = np.ascontiguousarray(lw.grids[j], dtype=np.float64)
            keep.append(g)
            d.coords[j] = g.ctypes.data_as(C.POINTER(C.c_double))
        for (f, j, s), e in lw.bcs.items():
            b = d.bc[f][j][s]
            b.kind = e["kind"]
            b.prog = e["prog"]
            b.op = e["op"]
            b.a, b.b, b.g = e["a"], e["b"], e["g"]
            b.extrap = e.get("extrap", 0)
            b.iop = e.get("iop", 0)
        # operators and the weight pool
        pool: List[float] = []
        ops = (L.mol_op1d * max(1, len(lw.ops)))()
        for i, o in enumerate(lw.ops):
            r = ops[i]
            r.L, r.omin, r.nlo, r.bLlo, r.nhi, r.bLhi, r.hi_base = o.L, o.omin, o.nlo, o.bLlo, o.nhi, o.bLhi, o.hi_base
            r.w_int = len(pool)
            if o.rows is not None:          # nonuniform grid: one interior row per interior point
                r.nrows = len(o.rows)
                for w in o.rows:
                    pool += list(w)
            else:
                pool += list(o.interior)
            r.w_lo = len(pool)
            for w in o.low:
                pool += list(w)
            r.w_hi = len(pool)
            for w in o.high:
                pool += list(w)
        self.weights = np.array(pool if pool else [0.0], dtype=np.float64)
        keep += [ops, self.weights]
        d.nops = len(lw.ops)
        d.ops = C.cast(ops, C.POINTER(L.mol_op1d))
        d.nweights = len(pool)
        d.weights = self.weights.ctypes.data_as(C.POINTER(C.c_double))
        terms = (L.mol_term * max(1, len(lw.terms)))()
        for i, t in enumerate(lw.terms):
            r = terms[i]
            r.kind = t["kind"]
            r.field = t["field"]
            r.dim = t["dim"]
            r.dim2 = t.get("dim2", 0)
            r.op = t.get("op", 0)
            r.op2 = t.get("op2", 0)
            r.op3 = t.get("op3", 0)
            r.prog = t.get("prog", -1)
            r.aux0 = t.get("aux0", 0)
            r.eps = t.get("eps", 0.0)
            r.dx = t.get("dx", 0.0)
            r.variant = t.get("variant", 0)
        keep.append(terms)
        d.nterms = len(lw.terms)
        d.terms = C.cast(terms, C.POINTER(L.mol_term))
        code = []
        ranges = []
        for prog in lw.programs:
            ranges += [len(code), len(prog)]
            code += prog
        instrs = (L.mol_instr * max(1, len(code)))()
        for i, (op, dst, a, b, c, imm) in enumerate(code):
            r = instrs[i]
            r.op, r.dst, r.a, r.b, r.c, r.imm = op, dst, a, b, c, imm
        rng = (C.c_int32 * max(1, len(ranges)))(*ranges)
        keep += [instrs, rng]
        d.ninstr = len(code)
        d.code = C.cast(instrs, C.POINTER(L.mol_instr))
        d.nprogs = len(lw.programs)
        d.prog_ranges = C.cast(rng, C.POINTER(C.c_int32))
        d.cell_prog = lw.cell_prog
        self.consts = np.array(lw.consts if lw.consts else [0.0], dtype=np.float64)
        keep.append(self.consts)
        d.nconsts = len(lw.consts)
        d.consts = self.consts.ctypes.data_as(C.POINTER(C.c_double))
        auxp = (C.POINTER(C.c_double) * max(1, len(lw.aux)))()
        auxl = (C.c_int64 * max(1, len(lw.aux)))()
        for i, a in enumerate(lw.aux):
            auxp[i] = a.ctypes.data_as(C.POINTER(C.c_double))
            auxl[i] = a.size
        keep += [auxp, auxl]
        d.naux = len(lw.aux)
        d.aux = C.cast(auxp, C.POINTER(C.POINTER(C.c_double)))
        d.aux_len = C.cast(auxl, C.POINTER(C.c_int64))
        self.params = np.ascontiguousarray(lw.param_values if len(lw.param_values) else np.zeros(1))
        keep.append(self.params)
        d.params = self.params.ctypes.data_as(C.POINTER(C.c_double))
        d.flags = 0
        self.desc = d
        self._keep = keep
