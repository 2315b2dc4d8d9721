"""Oracle restatement of MethodOfLines.jl's semi-discretisation (CPU, numpy).

Given a problem *spec* (the plain-data form of a ``PDESystem`` plus the
``MOLFiniteDifference`` options, see ``molgpu.symbolic.PDESystem.to_spec``), this
module rebuilds what ``discretize`` would produce: the grid, the unknown set,
the observed boundary values and the right-hand side ``f(du, u, p, t)``.  Every
scheme follows the reference file cited in its docstring; nothing here is
shared with the GPU product.

Test infrastructure only.  The product package never imports this module.
"""
from __future__ import annotations

import math
from fractions import Fraction
from typing import Dict, List, Tuple

import numpy as np

from .weno_nonuniform import taps_and_target, weno_f_nonuniform
from .fornberg import (boundary_interpolator_extrapolator, complete_centered_difference,
                       complete_centered_difference_nonuniform, complete_half_centered_difference,
                       complete_half_centered_difference_nonuniform,
                       complete_upwind_difference_nonuniform,
                       complete_upwind_difference)

# --------------------------------------------------------------------------------------
# grids: src/discretization/discretize_vars.jl:219-285 (Julia float ranges)
# --------------------------------------------------------------------------------------


def _rat(x: float):
    """Continued-fraction rational approximation with |p|,|q| <= 2^24 (Julia ``Base.rat``)."""
    y = x
    a, d = 1, 1
    b, c = 0, 0
    m = 2 ** 24
    while abs(y) <= m:
        f = int(y)  # trunc
        y -= f
        a, c = f * a + c, a
        b, d = f * b + d, b
        if max(abs(a), abs(b)) > m:
            return c, d
        if b != 0 and float(a) / float(b) == x:
            break
        if y == 0:
            break
        y = 1.0 / y
    return a, b


def julia_float_range(start: float, step: float, stop: float) -> np.ndarray:
    """Elements of Julia's ``start:step:stop`` for Float64 (rational path, else literal path)."""
    sn, sd = _rat(step)
    if sd != 0 and float(sn) / float(sd) == step:
        an, ad = _rat(start)
        on, od = _rat(stop)
        if ad != 0 and od != 0 and float(an) / float(ad) == start and float(on) / float(od) == stop:
            den = ad * sd // math.gcd(ad, sd)
            a_n = round(start * den)
            s_n = round(step * den)
            ln = max(0, (den * on - od * a_n + s_n * od) // (s_n * od))
            last = float(Fraction(a_n + (ln - 1) * s_n, den))
            nxt = float(Fraction(a_n + ln * s_n, den))
            if start <= last <= stop + step / 2 and not (start <= nxt <= stop):
                return np.array([float(Fraction(a_n + k * s_n, den)) for k in range(ln)])
    lf = (stop - start) / step
    if lf < 0:
        ln = 0
    elif lf == 0:
        ln = 1
    else:
        ln = int(round(lf)) + 1
        stop2 = start + (ln - 1) * step
        ln -= int(start < stop < stop2) + int(start > stop > stop2)
    fs, fst = Fraction(start), Fraction(step)
    return np.array([float(fs + k * fst) for k in range(ln)])


def make_grid(lo: float, hi: float, dx_spec) -> Tuple[np.ndarray, float, bool]:
    """``discretize_space`` + ``prepare_dx`` for a center-aligned grid
    (discretize_vars.jl:218-233, :283-285): (points, step, uniform).  A step that does not
    reach ``hi`` gets ``hi`` appended, and a grid given as points is taken as it is (with
    ``hi`` appended the same way); both are Vectors, whose operators the reference builds
    from the points (differential_discretizer.jl:45-58)."""
    if isinstance(dx_spec, (int, np.integer)) and not isinstance(dx_spec, bool):
        dx = (hi - lo) / (int(dx_spec) - 1)
    elif isinstance(dx_spec, (float, np.floating)):
        dx = float(dx_spec)
    else:
        g = np.array([float(v) for v in dx_spec])
        if g[-1] != hi:
            g = np.append(g, hi)
        return g, float("nan"), False
    g = julia_float_range(lo, dx, hi)
    if g[-1] != hi:
        return np.append(g, hi), dx, False
    return g, dx, True


def make_edge_grid(lo: float, hi: float, dx_spec) -> Tuple[np.ndarray, float, bool]:
    """``generate_grid`` for EdgeAlignedGrid (discretize_vars.jl:373-390) on a StepRangeLen
    axis: ``(lo - dx/2):dx:(hi + dx/2)``; an integer is a number of cells (:284)."""
    if isinstance(dx_spec, (int, np.integer)) and not isinstance(dx_spec, bool):
        dx = (hi - lo) / int(dx_spec)
    else:
        dx = float(dx_spec)
    axis = julia_float_range(lo, dx, hi)
    if axis[-1] != hi:
        raise NotImplementedError("oracle: edge-aligned grid of midpoints")
    return julia_float_range(lo - dx / 2, dx, hi + dx / 2), dx, True


# --------------------------------------------------------------------------------------
# tap selection: centered_difference.jl:5-30, upwind_difference.jl:1-28,
# half_offset_centred_difference.jl:9-37, interface_boundary.jl:26-42
# --------------------------------------------------------------------------------------


def wrap_periodic(i: int, l: int) -> int:
    """``_wrapperiodic``: u[1] == u[l]; index <= 1 shifts up by l-1, index > l shifts down."""
    if i <= 1:
        return i + (l - 1)
    if i > l:
        return i - (l - 1)
    return i


def central_taps(D, i: int, n: int, periodic: bool):
    """Weights and (1-based) taps of ``central_difference_weights_and_stencil`` at index i."""
    bpc = D.boundary_point_count
    bL = D.boundary_stencil_length
    if i <= bpc and not periodic:
        return list(D.low_boundary_coefs[i - 1]), [1 + k for k in range(bL)]
    if i > n - bpc and not periodic:
        return list(D.high_boundary_coefs[n - i]), [n - bL + 1 + k for k in range(bL)]
    half = D.stencil_length // 2
    taps = [i + k for k in range(-half, half + 1)]
    if D.kind == "centered_nonuniform":   # centered_difference.jl:51-53: the point's own row
        assert not periodic, "interface boundaries are not supported on nonuniform dimensions"
        return list(D.stencil_coefs[i - bpc - 1]), taps
    if periodic:
        taps = [wrap_periodic(t, n) for t in taps]
    return list(D.stencil_coefs), taps


def upwind_taps(D, i: int, n: int, periodic: bool, ispositive: bool):
    """``_upwind_difference`` (uniform dx, upwind_difference.jl:1-28; a nonuniform grid without
    interfaces, :131-162)."""
    L = D.stencil_length
    bL = D.boundary_stencil_length
    if D.kind == "upwind_nonuniform":
        assert not periodic, "interfaces on nonuniform upwind dimensions are not restated"
        if not ispositive:
            if i > n - D.boundary_point_count:
                return list(D.high_boundary_coefs[n - i]), [n - bL + 1 + k for k in range(bL)]
            return list(D.stencil_coefs[i - 1]), [i + k for k in range(0, L)]
        # D.offside is 0 as the reference returns the operator: never the low rows
        return list(D.stencil_coefs[i - 1]), [i + k for k in range(-L + 1, 1)]
    if not ispositive:
        if i > n - D.boundary_point_count and not periodic:
            return list(D.high_boundary_coefs[n - i]), [n - bL + 1 + k for k in range(bL)]
        taps = [i + k for k in range(0, L)]
    else:
        if i <= D.offside and not periodic:
            return list(D.low_boundary_coefs[i - 1]), [1 + k for k in range(bL)]
        taps = [i + k for k in range(-L + 1, 1)]
    if periodic:
        taps = [wrap_periodic(t, n) for t in taps]
    return list(D.stencil_coefs), taps


def half_offset_taps(D, i: int, n: int, periodic: bool, length: int = 0, wrap: bool = True):
    """``get_half_offset_weights_and_stencil``; taps are *not* wrapped here (callers wrap)."""
    ln = n if length == 0 else length
    bpc = D.boundary_point_count
    bL = D.boundary_stencil_length
    if i <= bpc and not periodic:
        return list(D.low_boundary_coefs[i - 1]), [1 + k for k in range(bL)]
    if i > ln - bpc and not periodic:
        return list(D.high_boundary_coefs[ln - i - 1]), [ln - bL + 1 + k for k in range(bL)]
    h = D.stencil_length // 2
    taps = [i + k for k in range(1 - h, h + 1)]
    if D.kind == "half_nonuniform":     # half_offset_centred_difference.jl:39-69: the point's own row
        assert not periodic, "interface boundaries are not supported on nonuniform dimensions"
        return list(D.stencil_coefs[i - bpc - 1]), taps
    return list(D.stencil_coefs), taps


# --------------------------------------------------------------------------------------
# expression helpers
# --------------------------------------------------------------------------------------

_FN = {
    "sin": np.sin, "cos": np.cos, "tan": np.tan, "exp": np.exp, "log": np.log,
    "sqrt": np.sqrt, "abs": np.abs, "tanh": np.tanh, "sinh": np.sinh, "cosh": np.cosh,
    "atan": np.arctan,
}


def _powi(a, n: int):
    """Integer powers as Julia's literal_pow gives them for small n: x*x, x*x*x."""
    if n == 0:
        return np.ones_like(a) if isinstance(a, np.ndarray) else 1.0
    if n == 1:
        return a
    if n == 2:
        return a * a
    if n == 3:
        return a * a * a
    if n == -1:
        return 1.0 / a
    if n == -2:
        return 1.0 / (a * a)
    return np.power(a, float(n))


def _is_num(t):
    return t[0] == "num"


def _split_add(t, sign=1.0):
    """Top-level additive terms with the sign pushed into each term (Symbolics' Add)."""
    k = t[0]
    if k == "add":
        out = []
        for a in t[1:]:
            out += _split_add(a, sign)
        return out
    if k == "sub":
        return _split_add(t[1], sign) + _split_add(t[2], -sign)
    if k == "neg":
        return _split_add(t[1], -sign)
    return [(sign, t)]


def _deriv_orders(t, x):
    """Orders of the derivatives along x anywhere in the expression (``d_orders``)."""
    out = set()
    if isinstance(t, tuple) and t:
        if t[0] == "D" and t[1] == x:
            out.add(t[2])
        for a in t[1:]:
            if isinstance(a, tuple):
                out |= _deriv_orders(a, x)
    return out


def _split_mul(t):
    """Multiplicative factors (numerator list, denominator list)."""
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


def _is_field_deriv(t, order=None):
    return (t[0] == "D" and t[3][0] == "field" and (order is None or t[2] == order))


class OracleProblem:
    """The reference's discretisation of one PDE system, restated on the CPU.

    Layout of the unknown vector: fields in declaration order, each field's
    interior box flattened with the first spatial variable fastest (the order
    of ``unknowns`` in the reference's generated code, e.g.
    ``docs/src/generated/bruss_code.md``).
    """

    def __init__(self, spec: dict):
        self.spec = spec
        self.ivs: List[str] = list(spec["ivs"])
        self.nd = len(self.ivs)
        self.fields: List[str] = list(spec["fields"])
        self.param_names = [p[0] for p in spec.get("params", [])]
        self.param_values = np.array([float(p[1]) for p in spec.get("params", [])], dtype=np.float64)
        self.functions = spec.get("functions", {})
        disc = spec["disc"]
        self.order = int(disc.get("approx_order", 2))
        adv = disc.get("advection", ["upwind", 1])
        self.adv_kind = adv[0]
        self.adv_param = adv[1]
        # grids
        self.grid = []
        self.dx = []
        self.uniform = []
        self.edge = disc.get("grid_align", "center") == "edge"
        for x in self.ivs:
            lo, hi = spec["domain"][x]
            if self.edge:
                g, dx, uni = make_edge_grid(float(lo), float(hi), disc["dxs"][x])
            else:
                g, dx, uni = make_grid(float(lo), float(hi), disc["dxs"][x])
            self.uniform.append(uni)
            self.grid.append(g)
            self.dx.append(dx)
        self.npts = [len(g) for g in self.grid]
        # boundary conditions: per field, per dim: {"periodic": bool, "lo": bc, "hi": bc}
        self.bc = {f: [{"periodic": False, "lo": None, "hi": None} for _ in range(self.nd)]
                   for f in self.fields}
        for b in spec.get("bcs", []):
            f, j = b["field"], self.ivs.index(b["iv"])
            if b["kind"] == "periodic":
                self.bc[f][j]["periodic"] = True
            else:
                self.bc[f][j][b["side"]] = b
        # interior boxes: interior_map.jl:1-10 (clip one point per truncating boundary;
        # a periodic pair clips only the lower end) and :53-139 (stencil extents)
        self.lower = {}
        self.upper = {}
        for f in self.fields:
            lo = [0] * self.nd
            up = [0] * self.nd
            for j in range(self.nd):
                bj = self.bc[f][j]
                if bj["periodic"]:
                    lo[j] += 1
                else:
                    lo[j] += int(bj["lo"] is not None)
                    up[j] += int(bj["hi"] is not None)
            self.lower[f] = lo
            self.upper[f] = up
        # stencil extents (interior_map.jl:83-90, :117-139): the advection scheme's extent
        # along every dimension where the equation has a first derivative and no periodic
        # boundary; WENO reaches 2 on a uniform grid and 0 on a nonuniform one (WENO.jl:94-95).
        # The points between the boundary row and the interior are then extrapolated
        # (generate_extrap_eqs!, generate_bc_eqs.jl:336-392).
        self.clip_lower = {f: list(self.lower[f]) for f in self.fields}
        self.clip_upper = {f: list(self.upper[f]) for f in self.fields}
        if self.adv_kind == "weno":
            for f in self.fields:
                for j, x in enumerate(self.ivs):
                    if self.bc[f][j]["periodic"] or 1 not in _deriv_orders(spec["eqs"][f], x):
                        continue
                    ext = 2 if self.uniform[j] else 0
                    self.lower[f][j] = max(self.lower[f][j], ext)
                    self.upper[f][j] = max(self.upper[f][j], ext)
        self.shape = {f: tuple(self.npts[j] - self.lower[f][j] - self.upper[f][j] for j in range(self.nd))
                      for f in self.fields}
        self.size = {f: int(np.prod(self.shape[f])) for f in self.fields}
        self.offset = {}
        off = 0
        for f in self.fields:
            self.offset[f] = off
            off += self.size[f]
        self.n_unknowns = off
        self._ops = {}

    # ---------------------------------------------------------------- operators
    def op(self, kind: str, j: int, d: int, extra=None):
        key = (kind, j, d, extra)
        if key not in self._ops:
            dx = self.dx[j]
            if not self.uniform[j]:
                if kind == "centered":
                    D = complete_centered_difference_nonuniform(d, self.order, self.grid[j])
                elif kind == "wind_neg":
                    D = complete_upwind_difference_nonuniform(d, int(extra), self.grid[j], 0)
                elif kind == "wind_pos":
                    D = complete_upwind_difference_nonuniform(d, int(extra), self.grid[j], d + int(extra) - 1)
                elif kind == "half":
                    D = complete_half_centered_difference_nonuniform(d, self.order, self.grid[j])
                elif kind == "interp":
                    D = complete_half_centered_difference_nonuniform(0, max(4, self.order), self.grid[j])
                elif kind == "half_outer":
                    # differential_discretizer.jl:47-52: the outer operator of the nonlinear
                    # Laplacian is built on the midpoints of the grid
                    g = self.grid[j]
                    D = complete_half_centered_difference_nonuniform(
                        d, self.order, [(g[i + 1] + g[i]) / 2 for i in range(len(g) - 1)])
                else:
                    raise NotImplementedError(f"oracle: {kind} operators on a nonuniform grid")
            elif kind == "centered":
                D = complete_centered_difference(d, self.order, dx)
            elif kind == "wind_neg":        # windmap[1]: offside 0, used when !ispositive
                D = complete_upwind_difference(d, int(extra), dx, 0)
            elif kind == "wind_pos":        # windmap[2]: offside d+p-1
                D = complete_upwind_difference(d, int(extra), dx, d + int(extra) - 1)
            elif kind == "half":
                D = complete_half_centered_difference(d, self.order, dx)
            elif kind == "extrap":
                D = boundary_interpolator_extrapolator(max(6, self.order), dx)
            elif kind == "interp":
                D = complete_half_centered_difference(0, max(4, self.order), dx)
            else:
                raise ValueError(kind)
            self._ops[key] = D
        return self._ops[key]

    # ---------------------------------------------------------------- state maps
    def interior_index(self, f: str, j: int) -> np.ndarray:
        """1-based grid indices of field f's interior along dim j."""
        return np.arange(1 + self.lower[f][j], self.npts[j] - self.upper[f][j] + 1)

    def unpack(self, u: np.ndarray) -> Dict[str, np.ndarray]:
        out = {}
        for f in self.fields:
            out[f] = np.asarray(u[self.offset[f]:self.offset[f] + self.size[f]]).reshape(self.shape[f], order="F")
        return out

    def pack(self, d: Dict[str, np.ndarray]) -> np.ndarray:
        return np.concatenate([np.asarray(d[f]).reshape(-1, order="F") for f in self.fields])

    def coords_interior(self, f: str):
        idx = [self.interior_index(f, j) for j in range(self.nd)]
        return np.meshgrid(*[self.grid[j][idx[j] - 1] for j in range(self.nd)], indexing="ij")

    def initial_condition(self) -> np.ndarray:
        """u0 from the spec's initial conditions at the interior points (generate_ic_defaults.jl:1-27)."""
        parts = {}
        for f in self.fields:
            X = self.coords_interior(f)
            env = {"coords": {self.ivs[j]: X[j] for j in range(self.nd)}, "t": float(self.spec["domain"][self.spec["time"]][0])}
            v = self._eval_point(self.spec["ics"][f], env)
            parts[f] = np.broadcast_to(np.asarray(v, dtype=np.float64), self.shape[f]).copy()
        return self.pack(parts)

    def _eval_point(self, t, env):
        """Pointwise expression evaluation (no derivatives), IEEE op by op."""
        k = t[0]
        if k == "num":
            return t[1]
        if k == "param":
            return env["p"][self.param_names.index(t[1])]
        if k == "iv":
            return env["coords"][t[1]]
        if k == "t":
            return env["t"]
        if k == "field":
            return env["fields"][t[1]]
        if k == "add":
            acc = self._eval_point(t[1], env)
            for a in t[2:]:
                acc = acc + self._eval_point(a, env)
            return acc
        if k == "mul":
            acc = self._eval_point(t[1], env)
            for a in t[2:]:
                acc = acc * self._eval_point(a, env)
            return acc
        if k == "sub":
            return self._eval_point(t[1], env) - self._eval_point(t[2], env)
        if k == "neg":
            return -self._eval_point(t[1], env)
        if k == "div":
            return self._eval_point(t[1], env) / self._eval_point(t[2], env)
        if k == "pow":
            a = self._eval_point(t[1], env)
            if t[2][0] == "num" and float(t[2][1]).is_integer():
                return _powi(a, int(t[2][1]))
            return np.power(a, self._eval_point(t[2], env))
        if k == "fn":
            return _FN[t[1]](self._eval_point(t[2], env))
        if k == "call":
            args = [self._eval_point(a, env) for a in t[2:]]
            return self.functions[t[1]](*args)
        if k == "cmp":
            a = self._eval_point(t[2], env)
            b = self._eval_point(t[3], env)
            r = {"<=": np.less_equal, "<": np.less, ">=": np.greater_equal, ">": np.greater,
                 "==": np.equal}[t[1]](a, b)
            return np.asarray(r, dtype=np.float64) if isinstance(r, np.ndarray) else float(r)
        if k == "ifelse":
            c = self._eval_point(t[1], env)
            return np.where(np.asarray(c) != 0, self._eval_point(t[2], env), self._eval_point(t[3], env))
        if k == "D":
            return env["deriv"](t)
        raise ValueError(f"unsupported node {k}")

    # ---------------------------------------------------------------- full-grid values
    def full_arrays(self, u: np.ndarray, t: float, p: np.ndarray) -> Dict[str, np.ndarray]:
        """Every grid point's value: unknowns, periodic images, observed BC values, corners = 0.

        BC rows: ``generate_bc_eqs.jl:238-328`` (Robin/Neumann/Dirichlet with the one-sided
        centered table at the boundary index, solved for the boundary value), periodic rows
        ``:35-58`` (u[1] ~ u[l]) and corner rows ``:396-459`` (~ 0).
        """
        parts = self.unpack(u)
        full = {}
        for f in self.fields:
            F = np.zeros(self.npts, dtype=np.float64)
            sl = tuple(slice(self.lower[f][j], self.npts[j] - self.upper[f][j]) for j in range(self.nd))
            F[sl] = parts[f]
            full[f] = F
        for f in self.fields:
            F = full[f]
            for j in range(self.nd):
                bj = self.bc[f][j]
                if bj["periodic"]:
                    idx_src = [slice(None)] * self.nd
                    idx_dst = [slice(None)] * self.nd
                    idx_src[j] = self.npts[j] - 1
                    idx_dst[j] = 0
                    # only the interior of the other dimensions is defined this way;
                    # the other entries are overwritten below or are corners
                    F[tuple(idx_dst)] = F[tuple(idx_src)]
            for j in range(self.nd):
                for side in ("lo", "hi"):
                    b = self.bc[f][j][side]
                    if b is None:
                        continue
                    if self.edge:
                        self._fill_edge(F, f, j, side, b, t, p)
                    else:
                        self._fill_robin(F, f, j, side, b, t, p)
            for j in range(self.nd):
                self._fill_extrapolated(F, f, j)
            self._zero_corners(F, f)
        return full

    def _fill_extrapolated(self, F, f, j):
        """``generate_extrap_eqs!`` (generate_bc_eqs.jl:336-392): the points between the boundary
        row and the interior, on the interior's edge slice, are ``central_difference`` of the
        extrapolator ``BoundaryInterpolatorExtrapolator(max(6, order), dx)`` at that point."""
        n = self.npts[j]
        for side in ("lo", "hi"):
            ext = self.lower[f][j] if side == "lo" else self.upper[f][j]
            clip = self.clip_lower[f][j] if side == "lo" else self.clip_upper[f][j]
            if ext <= clip:
                continue
            if clip == 0:
                raise NotImplementedError("oracle: extrapolated points with no boundary row at that end")
            Dx = self.op("extrap", j, 0)
            sl = self._other_interior_slices(f, j)
            for m in range(clip + 1, ext + 1):
                i = m if side == "lo" else n + 1 - m
                w, taps = central_taps(Dx, i, n, False)
                acc = None
                for wk, tp in zip(w, taps):
                    if wk == 0.0:
                        continue
                    s = list(sl)
                    s[j] = tp - 1
                    term = wk * F[tuple(s)]
                    acc = term if acc is None else acc + term
                s = list(sl)
                s[j] = i - 1
                F[tuple(s)] = acc

    def solution_arrays(self, u: np.ndarray, t: float, p: np.ndarray) -> Dict[str, np.ndarray]:
        """The arrays behind sol[u(t, x)] (interface/solution/timedep.jl:19-80): every discrete
        variable, the observed ones from their equations.  Periodic rows (generate_bc_eqs.jl:
        35-58) and boundary rows cover only the interior's edge slices, so a point outside the
        interior box in two or more dimensions, periodic images included, is a corner row ~ 0
        (generate_bc_eqs.jl:396-459); ``full_arrays`` instead fills such points of two periodic
        dimensions with the wrapped value, which is what the right-hand side's wrapped taps
        read."""
        full = self.full_arrays(u, t, p)
        for f in self.fields:
            outside = np.zeros(self.npts, dtype=np.int32)
            for j in range(self.nd):
                idx = np.arange(1, self.npts[j] + 1)
                m = (idx <= self.lower[f][j]) | (idx > self.npts[j] - self.upper[f][j])
                shp = [1] * self.nd
                shp[j] = self.npts[j]
                outside = outside + m.reshape(shp)
            full[f][outside >= 2] = 0.0
        return full

    def _other_interior_slices(self, f, j):
        sl = []
        for k in range(self.nd):
            if k == j:
                sl.append(None)
            else:
                sl.append(slice(self.lower[f][k], self.npts[k] - self.upper[f][k]))
        return sl

    def _fill_robin(self, F, f, j, side, b, t, p):
        n = self.npts[j]
        D1 = self.op("centered", j, 1)
        i = 1 if side == "lo" else n
        w, taps = central_taps(D1, i, n, False)
        sl = self._other_interior_slices(f, j)
        def at(idx):
            s = list(sl)
            s[j] = idx - 1
            return tuple(s)
        # coordinates on the face (other dims at their interior points)
        cs = {}
        for k in range(self.nd):
            if k == j:
                cs[self.ivs[k]] = self.grid[k][i - 1]
            else:
                g = self.grid[k][sl[k]]
                shp = [1] * self.nd
                shp[k] = len(g)
                cs[self.ivs[k]] = g.reshape([s for kk, s in enumerate(shp) if kk != j])
        env = {"coords": cs, "t": t, "p": p}
        a = self._eval_point(b["a"], env)
        bb = self._eval_point(b["b"], env)
        g = self._eval_point(b["g"], env)
        # a*u_b + b*(sum_k w_k u_k) = g, solved for u_b
        k_b = taps.index(i)
        acc = None
        for k, tp in enumerate(taps):
            if k == k_b:
                continue
            term = w[k] * F[at(tp)]
            acc = term if acc is None else acc + term
        F[at(i)] = (g - bb * acc) / (a + bb * w[k_b])

    def _fill_edge(self, F, f, j, side, b, t, p):
        """Edge-aligned boundary row (``boundary_value_maps`` for EdgeAlignedGrid,
        generate_bc_eqs.jl:80-160): u and Dx(u) at the face become the half-offset
        interpolation (``interpmap``) and first derivative (``halfoffsetmap``) at index 1, or
        ``length - 1`` (``newindex(...; shift = true)``, MOL_utils.jl:75-97), and the equation
        a*u + b*Dx(u) = g is solved for the ghost point."""
        n = self.npts[j]
        pos = 1 if side == "lo" else n - 1
        ghost = 1 if side == "lo" else n
        wi, ti = half_offset_taps(self.op("interp", j, 0), pos, n, False)
        wd, td = half_offset_taps(self.op("half", j, 1), pos, n, False)
        sl = self._other_interior_slices(f, j)

        def at(idx):
            s = list(sl)
            s[j] = idx - 1
            return tuple(s)
        cs = {}
        for k in range(self.nd):
            if k == j:   # axiesvals (discretize_vars.jl:321-330): the domain's end, not the ghost
                cs[self.ivs[k]] = float(self.spec["domain"][self.ivs[k]][0 if side == "lo" else 1])
            else:
                g = self.grid[k][sl[k]]
                shp = [1] * self.nd
                shp[k] = len(g)
                cs[self.ivs[k]] = g.reshape([s for kk, s in enumerate(shp) if kk != j])
        env = {"coords": cs, "t": t, "p": p}
        a = self._eval_point(b["a"], env)
        bb = self._eval_point(b["b"], env)
        g = self._eval_point(b["g"], env)
        si = sd = 0.0
        ci = cd = 0.0
        for w, tp in zip(wi, ti):
            if tp == ghost:
                ci = w
            else:
                si = si + w * F[at(tp)]
        for w, tp in zip(wd, td):
            if tp == ghost:
                cd = w
            else:
                sd = sd + w * F[at(tp)]
        F[at(ghost)] = (g - a * si - bb * sd) / (a * ci + bb * cd)

    def _zero_corners(self, F, f):
        if self.nd < 2:
            return
        outside = np.zeros(self.npts, dtype=np.int32)
        for j in range(self.nd):
            idx = np.arange(1, self.npts[j] + 1)
            if self.bc[f][j]["periodic"]:
                m = np.zeros(self.npts[j], dtype=bool)
            else:
                m = (idx <= self.lower[f][j]) | (idx > self.npts[j] - self.upper[f][j])
            shp = [1] * self.nd
            shp[j] = self.npts[j]
            outside = outside + m.reshape(shp)
        F[outside >= 2] = 0.0

    # ---------------------------------------------------------------- RHS
    def rhs(self, u: np.ndarray, t: float, p=None) -> np.ndarray:
        """``f(du, u, p, t)`` of the reference's generated ODE function."""
        p = self.param_values if p is None else np.asarray(p, dtype=np.float64)
        full = self.full_arrays(np.asarray(u, dtype=np.float64), t, p)
        out = {}
        for f in self.fields:
            out[f] = self._eval_rhs(f, full, t, p)
        return self.pack(out)

    def _eval_rhs(self, f, full, t, p):
        X = self.coords_interior(f)
        sl = tuple(slice(self.lower[f][j], self.npts[j] - self.upper[f][j]) for j in range(self.nd))
        env = {"coords": {self.ivs[j]: X[j] for j in range(self.nd)}, "t": t, "p": p,
               "fields": {g: full[g][sl] for g in self.fields}}
        env["deriv"] = lambda node: self._deriv(node, f, full, env, None)
        acc = None
        for sign, term in _split_add(self.spec["eqs"][f]):
            v = self._eval_term(term, sign, f, full, env)
            acc = v if acc is None else acc + v
        return np.broadcast_to(acc, self.shape[f]).copy()

    def _eval_term(self, term, sign, f, full, env):
        """One additive term of the right-hand side (sign already pushed in).

        Upwinding (upwind_difference.jl:184-199, 201-303): a term ``kappa * Dx^d(u)`` with odd d on
        the right-hand side is ``(-kappa) * Dx^d(u)`` on the cardinalised left-hand side; the reference
        takes the backward stencil when that coefficient is > 0, the forward one otherwise.
        """
        num, den = _split_mul(term)
        sph = self._spherical(num, den, f, full, env)
        if sph is not None:
            return -sph if sign < 0 else sph
        odd = [k for k, a in enumerate(num) if _is_field_deriv(a) and a[2] % 2 == 1
               and not (self.adv_kind == "weno" and a[2] == 1)]
        if odd:
            kd = odd[0]
            others = num[:kd] + num[kd + 1:]
            kap = None
            for a in others:
                v = self._eval_point(a, env)
                kap = v if kap is None else kap * v
            for dnode in den:
                v = self._eval_point(dnode, env)
                kap = (1.0 / v) if kap is None else kap / v
            if kap is None:
                kap = 1.0
            if sign < 0:
                kap = -kap
            c = -kap                                      # coefficient on the left-hand side
            dpos = self._deriv(num[kd], f, full, env, True)
            dneg = self._deriv(num[kd], f, full, env, False)
            lhs = np.where(c > 0, c * dpos, c * dneg)
            return -lhs
        v = self._eval_point(term, env)
        return -v if sign < 0 else v

    def _spherical(self, num, den, f, full, env):
        """``generate_spherical_diffusion_rules`` / ``spherical_diffusion``
        (spherical_laplacian.jl:10-40, 42-130).

        A product whose only denominator is r^2 and one of whose factors is Dr(inner), inner a
        product holding r^2 and Dr(u), is rewritten: the other outer factors times
        spherical_diffusion(innerexpr), innerexpr the inner product without r^2 and Dr(u).  As
        the reference writes it, spherical_diffusion is innerexpr at the point times
        (D1(u) / r + cartesian_nonlinear_laplacian(innerexpr)), D1 the centered first
        derivative; at a point with |r| <= 1e-6 it is 6 innerexpr D2(u).  Returns None when
        the term does not have that form."""
        for kd, a in enumerate(num):
            if a[0] != "D" or a[2] != 1 or a[3][0] == "field":
                continue
            x = a[1]
            r2 = ("pow", ("iv", x), ("num", 2.0))
            if den != [r2]:
                continue
            inum, iden = _split_mul(a[3])
            if iden or inum.count(r2) != 1:
                continue
            ks = [k for k, q in enumerate(inum) if q[0] == "D" and q[1] == x and q[2] == 1 and q[3][0] == "field"]
            if len(ks) != 1:
                continue
            g = inum[ks[0]][3][1]
            coef = [q for k, q in enumerate(inum) if k != ks[0] and q != r2]
            j = self.ivs.index(x)
            r = self.coords_interior(f)[j]
            here = 1.0
            for c in coef:
                here = here * self._eval_point(c, env)
            d1 = self._linear(full[g], f, j, "centered", 1)
            nll = self._nonlinlap(coef, [], g, f, j, full, env)
            at0 = np.abs(r) <= 1e-6
            with np.errstate(divide="ignore", invalid="ignore"):
                v = here * (d1 / r + nll)
            if np.any(at0):
                v = np.where(at0, 6 * here * self._linear(full[g], f, j, "centered", 2), v)
            for k, q in enumerate(num):
                if k != kd:
                    v = self._eval_point(q, env) * v
            return v
        return None

    def _deriv(self, node, f, full, env, ispositive):
        _, x, d, arg = node
        j = self.ivs.index(x)
        if arg[0] == "field":
            g = arg[1]
            if d % 2 == 0:
                return self._linear(full[g], f, j, "centered", d)
            if self.adv_kind == "weno" and d == 1:
                return self._weno(full[g], f, j)
            return self._linear(full[g], f, j, "wind", d, True if ispositive is None else ispositive)
        if arg[0] == "D" and d == 1 and arg[2] == 1 and arg[3][0] == "field":
            k = self.ivs.index(arg[1])
            return self._mixed(full[arg[3][1]], f, j, k)
        # nonlinear laplacian: Dx(a * Dx(u))  (nonlinear_laplacian.jl:149-290)
        if d == 1:
            num, den = _split_mul(arg)
            ks = [k for k, a in enumerate(num) if a[0] == "D" and a[1] == x and a[2] == 1 and a[3][0] == "field"]
            if ks:
                inner = num[ks[0]]
                coef = num[:ks[0]] + num[ks[0] + 1:]
                return self._nonlinlap(coef, den, inner[3][1], f, j, full, env)
        raise NotImplementedError(f"derivative form not supported by the oracle: {node}")

    def _gather_1d(self, F, f, j, rows):
        """sum_k w_k F[tap_k] along dim j for each interior index; rows: list of (weights, taps)."""
        sl = [slice(self.lower[f][k], self.npts[k] - self.upper[f][k]) for k in range(self.nd)]
        out = []
        for (w, taps) in rows:
            acc = None
            for wk, tk in zip(w, taps):
                s = list(sl)
                s[j] = tk - 1
                term = wk * F[tuple(s)]
                acc = term if acc is None else acc + term
            out.append(acc)
        return np.stack(out, axis=j)

    def _linear(self, F, f, j, kind, d, ispositive=None):
        n = self.npts[j]
        per = self.bc[f][j]["periodic"]
        rows = []
        if kind == "centered":
            D = self.op("centered", j, d)
            for i in self.interior_index(f, j):
                rows.append(central_taps(D, int(i), n, per))
        else:
            p = self.adv_param if self.adv_kind == "upwind" else 1
            if ispositive:
                D = self.op("wind_pos", j, d, p)
            else:
                D = self.op("wind_neg", j, d, p)
            for i in self.interior_index(f, j):
                rows.append(upwind_taps(D, int(i), n, per, ispositive))
        return self._gather_1d(F, f, j, rows)

    def _mixed(self, F, f, j, k):
        """``mixed_central_difference`` (2nd_order_mixed_deriv.jl:5-22)."""
        Dx = self.op("centered", j, 1)
        Dy = self.op("centered", k, 1)
        nj, nk = self.npts[j], self.npts[k]
        pj, pk = self.bc[f][j]["periodic"], self.bc[f][k]["periodic"]
        ij = self.interior_index(f, j)
        ik = self.interior_index(f, k)

        def table(D, idxs, n, per):
            rows = [central_taps(D, int(i), n, per) for i in idxs]
            Lm = max(len(r[0]) for r in rows)
            W = np.zeros((len(rows), Lm))
            T = np.ones((len(rows), Lm), dtype=np.int64)
            for r, (w, taps) in enumerate(rows):
                W[r, :len(w)] = w
                T[r, :len(taps)] = taps
            return W, T

        Wx, Tx = table(Dx, ij, nj, pj)
        Wy, Ty = table(Dy, ik, nk, pk)
        # restrict the other dimensions to the interior, keep j and k full
        sl = [slice(self.lower[f][m], self.npts[m] - self.upper[f][m]) if m not in (j, k) else slice(None)
              for m in range(self.nd)]
        G = F[tuple(sl)]
        out = np.zeros(self.shape[f])
        acc_started = np.zeros(1, dtype=bool)
        for a in range(Wx.shape[1]):
            Ga = np.take(G, Tx[:, a] - 1, axis=j)
            for b in range(Wy.shape[1]):
                Gab = np.take(Ga, Ty[:, b] - 1, axis=k)
                shp = [1] * self.nd
                shp[j] = len(ij)
                wa = Wx[:, a].reshape(shp)
                shp = [1] * self.nd
                shp[k] = len(ik)
                wb = Wy[:, b].reshape(shp)
                term = wa * wb * Gab
                out = term if not acc_started[0] else out + term
                acc_started[0] = True
        return out

    def _weno(self, F, f, j):
        """``weno_f_uniform`` (WENO.jl:6-57) with taps from ``get_f_taps_coords`` (function_scheme.jl:1-34)."""
        n = self.npts[j]
        per = self.bc[f][j]["periodic"]
        idx = self.interior_index(f, j)
        if not self.uniform[j]:
            return self._weno_nonuniform(F, f, j)
        if not per and (idx[0] <= 2 or idx[-1] > n - 2):
            # get_f_taps_coords picks the near-wall functions there (function_scheme.jl:6-16)
            raise NotImplementedError("oracle: near-wall WENO stencils")
        eps = float(self.adv_param)
        dx = self.dx[j]
        sl = [slice(self.lower[f][k], self.npts[k] - self.upper[f][k]) for k in range(self.nd)]
        taps = [[wrap_periodic(int(i) + o, n) if per else int(i) + o for i in idx] for o in (-2, -1, 0, 1, 2)]
        def tap(o):
            s = list(sl)
            s[j] = np.array(taps[o + 2]) - 1
            return F[tuple(s)]
        u_m2, u_m1, u_0, u_p1, u_p2 = tap(-2), tap(-1), tap(0), tap(1), tap(2)
        return weno5(u_m2, u_m1, u_0, u_p1, u_p2, eps, dx)

    def _weno_nonuniform(self, F, f, j):
        """``function_scheme`` with the WENO scheme on a nonuniform dimension (function_scheme.jl:
        36-76): every point uses ``weno_f_nonuniform`` on the grid coordinates of its five taps,
        the two points at each end the one-sided targets (WENO.jl:84-85)."""
        n = self.npts[j]
        eps = float(self.adv_param)
        sl = [slice(self.lower[f][k], self.npts[k] - self.upper[f][k]) for k in range(self.nd)]
        out = []
        for i in self.interior_index(f, j):
            taps, tg = taps_and_target(int(i), n)
            vals = []
            for q in taps:
                s = list(sl)
                s[j] = q - 1
                vals.append(F[tuple(s)])
            xs = [self.grid[j][q - 1] for q in taps]
            out.append(weno_f_nonuniform(vals, eps, xs, tg))
        return np.stack(out, axis=j)

    def _nonlinlap(self, coef_num, coef_den, g, f, j, full, env):
        """``cartesian_nonlinear_laplacian`` (nonlinear_laplacian.jl:28-103)."""
        n = self.npts[j]
        per = self.bc[f][j]["periodic"]
        D_outer = self.op("half" if self.uniform[j] else "half_outer", j, 1)
        D_inner = self.op("half", j, 1)
        interp = self.op("interp", j, 0)
        cliplen = n - 1
        sl = [slice(self.lower[f][k], self.npts[k] - self.upper[f][k]) for k in range(self.nd)]
        wrapf = (lambda i: wrap_periodic(i, n)) if per else (lambda i: i)

        def line(F, i):
            s = list(sl)
            s[j] = i - 1
            return F[tuple(s)]

        Xint = self.coords_interior(f)
        results = []
        for II in self.interior_index(f, j):
            II = int(II)
            ow, ostencil = half_offset_taps(D_outer, II - 1, n, per, cliplen)
            acc = None
            for wo, I in zip(ow, ostencil):
                iw, itaps = half_offset_taps(interp, I, n, per)
                itaps = [wrapf(q) for q in itaps]
                dw, dtaps = half_offset_taps(D_inner, I, n, per)
                dtaps = [wrapf(q) for q in dtaps]
                # interpolated fields and coordinate at the half point
                fl = {}
                for h in self.fields:
                    a = None
                    for wk, tk in zip(iw, itaps):
                        term = wk * line(full[h], tk)
                        a = term if a is None else a + term
                    fl[h] = a
                # x => dot(weights, grid[x][wrapped taps]); the other ivs at the cell
                xc = None
                for wk, tk in zip(iw, itaps):
                    term = wk * self.grid[j][tk - 1]
                    xc = term if xc is None else xc + term
                coords = {}
                for k in range(self.nd):
                    if k == j:
                        coords[self.ivs[k]] = xc
                    else:
                        cut = tuple(slice(None) if kk != j else 0 for kk in range(self.nd))
                        coords[self.ivs[k]] = Xint[k][cut]
                fenv = {"coords": coords, "t": env["t"], "p": env["p"], "fields": fl}
                a = None
                for c in coef_num:
                    v = self._eval_point(c, fenv)
                    a = v if a is None else a * v
                for c in coef_den:
                    v = self._eval_point(c, fenv)
                    a = (1.0 / v) if a is None else a / v
                du = None
                for wk, tk in zip(dw, dtaps):
                    term = wk * line(full[g], tk)
                    du = term if du is None else du + term
                flux = du if a is None else a * du
                term = wo * flux
                acc = term if acc is None else acc + term
            results.append(acc)
        out = np.stack([np.broadcast_to(r, tuple(self.shape[f][k] for k in range(self.nd) if k != j))
                        for r in results], axis=j)
        return out


def weno5(u_m2, u_m1, u_0, u_p1, u_p2, eps, dx):
    """Jiang-Shu WENO5 node derivative exactly as ``weno_f_uniform`` writes it (WENO.jl:6-57)."""
    gm1, gm2, gm3 = 1 / 10, 3 / 5, 3 / 10
    b1 = 13 * (u_0 - 2 * u_p1 + u_p2) ** 2 / 12 + (3 * u_0 - 4 * u_p1 + u_p2) ** 2 / 4
    b2 = 13 * (u_m1 - 2 * u_0 + u_p1) ** 2 / 12 + (u_m1 - u_p1) ** 2 / 4
    b3 = 13 * (u_m2 - 2 * u_m1 + u_0) ** 2 / 12 + (u_m2 - 4 * u_m1 + 3 * u_0) ** 2 / 4
    wm1 = gm1 / (eps + b1) ** 2
    wm2 = gm2 / (eps + b2) ** 2
    wm3 = gm3 / (eps + b3) ** 2
    dm = wm1 + wm2 + wm3
    gp1, gp2, gp3 = 3 / 10, 3 / 5, 1 / 10
    wp1 = gp1 / (eps + b1) ** 2
    wp2 = gp2 / (eps + b2) ** 2
    wp3 = gp3 / (eps + b3) ** 2
    dp = wp1 + wp2 + wp3
    hm1 = (11 * u_0 - 7 * u_p1 + 2 * u_p2) / 6
    hm2 = (5 * u_0 - u_p1 + 2 * u_m1) / 6
    hm3 = (2 * u_0 + 5 * u_m1 - u_m2) / 6
    hp1 = (2 * u_0 + 5 * u_p1 - u_p2) / 6
    hp2 = (5 * u_0 + 2 * u_p1 - u_m1) / 6
    hp3 = (11 * u_0 - 7 * u_m1 + 2 * u_m2) / 6
    hp = (wp1 / dp) * hp1 + (wp2 / dp) * hp2 + (wp3 / dp) * hp3
    hm = (wm1 / dm) * hm1 + (wm2 / dm) * hm2 + (wm3 / dm) * hm3
    return (hp - hm) / dx
