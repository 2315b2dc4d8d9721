"""User-facing API mirroring MethodOfLines.jl / SciMLBase for the GPU hot path.

    disc = MOLFiniteDifference({x: dx, y: dy}, t, approx_order=2)
    prob = discretize(pdesys, disc)            # ODEProblem whose f calls mol_rhs
    prob.f(du, u, p, t)                        # the generated f!(du, u, p, t)
    sol = solve(prob, SSPRK33(), dt=1e-4)      # on-device stepping (mol_step_ssprk33)
    sol = solve(prob, Tsit5(), abstol=1e-10, reltol=1e-10)

Arrays may be numpy (host) or any object exposing ``data_ptr()`` on the GPU
(e.g. a torch CUDA tensor); the library detects which and stages host arrays.
"""
from __future__ import annotations

import ctypes as C
import math
import warnings
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib as L
from .lowering import Descriptor, Lowered, lower
from .symbolic import IV, Field, FieldApp, PDESystem


class UpwindScheme:
    """``UpwindScheme(order=1)`` (src/interface/scheme_types.jl:8-16)."""

    def __init__(self, order: int = 1):
        self.order = int(order)

    def spec(self):
        return ("upwind", self.order)


class WENOScheme:
    """``WENOScheme(; epsilon=1e-6)`` (src/discretization/schemes/WENO/WENO.jl:72-89)."""

    def __init__(self, epsilon: float = 1e-6):
        self.epsilon = float(epsilon)

    def spec(self):
        return ("weno", self.epsilon)


def _cospi(z: float) -> float:
    """cos(pi z), the argument reduced in z first (exact for the rationals chebyspace uses up to
    the last bit of the final cos/sin)."""
    r = math.fmod(abs(z), 2.0)
    if r > 1.0:
        r = 2.0 - r
    if r <= 0.25:
        return math.cos(math.pi * r)
    if r <= 0.75:
        return math.sin(math.pi * (0.5 - r))
    return -math.cos(math.pi * (1.0 - r))


def chebyspace(n: int, dom):
    """``chebyspace(N, dom)`` (src/MOL_utils.jl:112-123): N Chebyshev points of the first kind
    on the interval of ``dom = (x, Interval(a, b))`` in increasing order, the end points set
    to a and b; returns ``(x, points)`` for MOLFiniteDifference's dxs."""
    x, interval = dom
    a, b = float(interval.lo), float(interval.hi)
    pts = [(a + b) / 2 + (b - a) / 2 * _cospi((2 * k - 1) / (2 * n)) for k in range(1, n + 1)][::-1]
    pts[0], pts[-1] = a, b
    return x, np.array(pts)


center_align = "center"   # CenterAlignedGrid: the grid points are lo:dx:hi
edge_align = "edge"       # EdgeAlignedGrid: cell centres plus a ghost point beyond each end


class MOLFiniteDifference:
    """``MOLFiniteDifference(dxs, time; approx_order, advection_scheme, grid_align, ...)``
    (src/interface/MOLFiniteDifference.jl:31-76).  Only the options the GPU path honours are kept.

    ``dxs`` maps each spatial variable to a number of points (int), a step (float) or the
    grid's points (a sequence, a nonuniform grid: centered derivatives and boundary rows
    along it use per-point weights, centered_diff_weights.jl:77-153).

    GPU-backend keyword: ``stencil_form`` ("difference", the default, or "expanded") picks how
    a diffusion term with a coordinate-dependent coefficient, Dx(K(x) Dx(u)), is evaluated
    together with the constant-coefficient first-derivative terms beside it: from per-cell
    weights applied to differences u[tap] - u[cell] (the face form's rounding), or as one
    expanded sum of per-cell weights times unknowns (fewer FP64 operations; its rounding error
    relative to the result grows as the sum cancels, about 1 / (dx^2 u''/u) for diffusion)."""

    def __init__(self, dxs, time: Optional[IV] = None, approx_order: int = 2, advection_scheme=None,
                 grid_align: str = "center", **kwargs):
        self.dxs = {(k.name if isinstance(k, IV) else k): v for k, v in dict(dxs).items()}
        self.time = time
        self.approx_order = int(approx_order)
        if self.approx_order % 2 != 0:
            # MOLFiniteDifference.jl:56-58: a warning only; the odd order is kept and the
            # tables are built for it
            warnings.warn(f"Discretization approx_order must be even, rounding up to {self.approx_order + 1}")
        if self.approx_order < 1:
            raise ValueError("approx_order must be at least 1")
        self.advection_scheme = advection_scheme if advection_scheme is not None else UpwindScheme()
        self.grid_align = {"center_align": "center", "edge_align": "edge"}.get(grid_align, grid_align)
        if kwargs.get("upwind_order") is not None:
            # MOLFiniteDifference.jl:53-55: the keyword is accepted and has no effect
            warnings.warn("`upwind_order` no longer does anything; use advection_scheme=UpwindScheme(order)")
        self.stencil_form = kwargs.pop("stencil_form", "difference")
        if self.stencil_form not in ("difference", "expanded"):
            raise ValueError("stencil_form must be 'difference' or 'expanded'")
        self.kwargs = kwargs


def _ptr(a, n=None, name="array", f32=None, out=False):
    """(pointer, is_float32) of a numpy array or a CUDA tensor-like object.

    The library trusts the pointers it is given and reads or writes exactly the element
    counts its entry points document, so each argument is checked here first: float64 or
    float32 (``f32`` fixes which when given: the state's precision), contiguous, writable when
    ``out``, and exactly ``n`` elements when ``n`` is given and not 0."""
    if a is None:
        return None, None
    if hasattr(a, "data_ptr"):
        dt = str(getattr(a, "dtype", ""))
        is32 = dt.endswith("float32")
        if not (is32 or dt.endswith("float64")):
            raise TypeError(f"{name}: float64 or float32 elements expected, got {dt or type(a).__name__}")
        if hasattr(a, "is_contiguous") and not a.is_contiguous():
            raise ValueError(f"{name}: the array must be contiguous")
        size = int(a.numel()) if hasattr(a, "numel") else None
        ptr = C.c_void_p(a.data_ptr())
    else:
        if not isinstance(a, np.ndarray):
            raise TypeError(f"{name}: a numpy array or a CUDA tensor expected, got {type(a).__name__}")
        if a.dtype not in (np.float64, np.float32):
            raise TypeError(f"{name}: float64 or float32 elements expected, got {a.dtype}")
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError(f"{name}: the array must be contiguous")
        if out and not a.flags["WRITEABLE"]:
            raise ValueError(f"{name}: the array is written and must be writable")
        is32 = a.dtype == np.float32
        size = int(a.size)
        ptr = C.c_void_p(a.ctypes.data)
    if f32 is not None and bool(is32) != bool(f32):
        raise TypeError(f"{name}: {'float32' if f32 else 'float64'} elements expected, as the state has")
    if n and size is not None and size != n:          # n == 0: the pointer is not read
        raise ValueError(f"{name}: {n} elements expected, got {size}")
    return ptr, bool(is32)


class Plan:
    """Owner of one ``mol_plan``: the compiled GPU right-hand side and its steppers."""

    def __init__(self, lowered: Lowered, expand_stencils: bool = False):
        """``expand_stencils``: evaluate coefficient stencils as one expanded sum
        (MOL_FLAG_EXPAND_STENCILS) instead of on differences."""
        self.lowered = lowered
        self.desc = Descriptor(lowered)
        if expand_stencils:
            self.desc.desc.flags |= L.MOL_FLAG_EXPAND_STENCILS
        h = C.c_void_p()
        st = L.lib().mol_plan_create(C.byref(self.desc.desc), C.byref(h))
        self._h = h
        if st != 0:
            msg = (L.lib().mol_last_error(h) or b"").decode() if h.value else ""
            if h.value:
                L.lib().mol_plan_destroy(h)
            self._h = None
            raise L.MolError(st, msg)
        self.n = int(L.lib().mol_plan_n_unknowns(h))
        self.nparams = len(lowered.param_values)
        self.naux = int(sum(a.size for a in lowered.aux))

    def close(self):
        if getattr(self, "_h", None):
            L.lib().mol_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_handle: int):
        L.check(L.lib().mol_plan_set_stream(self._h, C.c_void_p(stream_handle)), self._h)

    def rhs(self, du, u, p=None, t: float = 0.0):
        """f!(du, u, p, t)."""
        pd, f32 = _ptr(du, self.n, "du", out=True)
        pu, _ = _ptr(u, self.n, "u", f32)
        pp, _ = _ptr(p, self.nparams, "p", f32)
        fn = L.lib().mol_rhs_f32state if f32 else L.lib().mol_rhs
        L.check(fn(self._h, pd, pu, pp, float(t)), self._h)
        return du

    def fill_grid(self, u, t: float = 0.0, p=None, out=None):
        """Every grid point of every field at state u and time t (``mol_fill_grid``): the
        unknowns plus the observed boundary values, extrapolated and ghost points, periodic
        images and corners, as sol[u(t, x)] holds them.  Host arrays give an array of shape
        (nfields, *npts); a device ``out`` (nfields * prod(npts) doubles) is filled in place."""
        lw = self.lowered
        per = int(np.prod(lw.npts))
        host_out = out is None or not hasattr(out, "data_ptr")
        buf = np.empty(len(lw.fields) * per) if out is None else out
        pu, _ = _ptr(u, self.n, "u", False)
        pp, _ = _ptr(p, self.nparams, "p", False)
        po, _ = _ptr(buf, len(lw.fields) * per, "out", False, out=True)
        L.check(L.lib().mol_fill_grid(self._h, pu, pp, float(t), po), self._h)
        if not host_out:
            return buf
        return np.stack([np.asarray(buf[k * per:(k + 1) * per]).reshape(lw.npts, order="F")
                         for k in range(len(lw.fields))])

    def step_ssprk33(self, u, dt: float, nsteps: int, t0: float = 0.0, p=None):
        pu, f32 = _ptr(u, self.n, "u", out=True)
        pp, _ = _ptr(p, self.nparams, "p", f32)
        fn = L.lib().mol_step_ssprk33_f32state if f32 else L.lib().mol_step_ssprk33
        L.check(fn(self._h, pu, pp, float(t0), float(dt), int(nsteps)), self._h)
        return u

    def check(self):
        """Waits for the plan's stream; raises MolError (MOL_ERR_NONFINITE) if an SSPRK33 step
        since the last check produced a NaN or Inf (steps on host arrays check themselves)."""
        L.check(L.lib().mol_plan_check(self._h), self._h)

    def step_ssprk33_noalloc(self, u, dt: float, nsteps: int, t0: float = 0.0, p=None):
        """SSPRK33 steps that allocate nothing (device arrays only, at most 2^20 unknowns)."""
        pu, _ = _ptr(u, self.n, "u", False, out=True)
        pp, _ = _ptr(p, self.nparams, "p", False)
        L.check(L.lib().mol_step_ssprk33_noalloc(self._h, pu, pp, float(t0), float(dt), int(nsteps)), self._h)
        return u

    def solve_tsit5(self, u, t0: float, t1: float, abstol: float, reltol: float, p=None, dt0: float = 0.0,
                    maxiters: int = 0):
        pu, _ = _ptr(u, self.n, "u", False, out=True)
        pp, _ = _ptr(p, self.nparams, "p", False)
        stats = L.mol_stats()
        L.check(L.lib().mol_solve_tsit5(self._h, pu, pp, float(t0), float(t1), float(abstol), float(reltol),
                                        float(dt0), int(maxiters), C.byref(stats)), self._h)
        return {"naccept": stats.naccept, "nreject": stats.nreject, "nf": stats.nf, "t": stats.t, "dt": stats.dt}

    @property
    def uses_codegen(self) -> bool:
        return bool(L.lib().mol_plan_uses_codegen(self._h))

    @property
    def coef_arrays(self) -> int:
        """Per-cell coefficient arrays of the plan's coefficient stencils (0: none)."""
        return int(L.lib().mol_plan_coef_arrays(self._h))

    @property
    def launch_config(self) -> dict:
        r, t, b = C.c_int32(), C.c_int32(), C.c_int32()
        L.check(L.lib().mol_plan_launch_config(self._h, C.byref(r), C.byref(t), C.byref(b)), self._h)
        return {"registers": r.value, "threads": t.value, "blocks": b.value}

    @property
    def generated_source(self) -> str:
        return (L.lib().mol_plan_codegen_source(self._h) or b"").decode()

    def vjp(self, lam, u, p=None, t: float = 0.0, lam_u=None, lam_p=None, lam_aux=None):
        n, npar, naux = self.n, self.nparams, self.naux
        L.check(L.lib().mol_rhs_vjp(self._h, _ptr(lam, n, "lam", False)[0], _ptr(u, n, "u", False)[0],
                                    _ptr(p, npar, "p", False)[0], float(t), _ptr(lam_u, n, "lam_u", False, True)[0],
                                    _ptr(lam_p, npar, "lam_p", False, True)[0],
                                    _ptr(lam_aux, naux, "lam_aux", False, True)[0]), self._h)

    def adjoint_ssprk33(self, u0, dt: float, nsteps: int, target, t0: float = 0.0, p=None, nsnap: int = 64,
                        loss_kind: int = L.LOSS_MISFIT, uT=None, dLdu0=None, dLdp=None, dLdaux=None):
        loss = np.zeros(1)
        nfw = C.c_int64(0)
        n, npar, naux = self.n, self.nparams, self.naux
        L.check(L.lib().mol_adjoint_ssprk33(self._h, _ptr(u0, n, "u0", False)[0], _ptr(p, npar, "p", False)[0],
                                            float(t0), float(dt), int(nsteps), int(nsnap), int(loss_kind),
                                            _ptr(target, n, "target", False)[0], _ptr(uT, n, "uT", False, True)[0],
                                            _ptr(loss)[0], _ptr(dLdu0, n, "dLdu0", False, True)[0],
                                            _ptr(dLdp, npar, "dLdp", False, True)[0],
                                            _ptr(dLdaux, naux, "dLdaux", False, True)[0], C.byref(nfw)), self._h)
        return float(loss[0]), int(nfw.value)

    @property
    def aux_sizes(self):
        return [a.size for a in self.lowered.aux]


class Batch:
    """An ensemble of instances of one PDE structure (uneven grids, own parameters) run by
    one persistent, graph-captured launch (``mol_batch_*``)."""

    def __init__(self, lowereds):
        self.lowereds = list(lowereds)
        self.descs = [Descriptor(lw) for lw in self.lowereds]
        n = len(self.descs)
        arr = (C.POINTER(L.mol_problem_desc) * n)(*[C.pointer(d.desc) for d in self.descs])
        h = C.c_void_p()
        st = L.lib().mol_batch_create(arr, n, C.byref(h))
        self._h = h
        if st != 0:
            msg = (L.lib().mol_batch_last_error(h) or b"").decode() if h.value else ""
            if h.value:
                L.lib().mol_batch_destroy(h)
            self._h = None
            raise L.MolError(st, msg)
        off = (C.c_int64 * (n + 1))()
        L.check(L.lib().mol_batch_offsets(h, off), batch=h)
        self.offsets = np.array(off[:], dtype=np.int64)
        self.n = n

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            L.lib().mol_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int):
        L.check(L.lib().mol_batch_set_stream(self._h, C.c_void_p(stream_handle)), batch=self._h)

    def pack(self, parts):
        return np.concatenate([np.asarray(p, dtype=np.float64) for p in parts])

    def step_ssprk33(self, u, dts, nsteps: int, t0: float = 0.0):
        pu, f32 = _ptr(u, int(self.offsets[-1]), "u", out=True)
        d = np.ascontiguousarray(dts, dtype=np.float64)
        if d.shape != (self.n,):
            raise ValueError(f"dts: one step per instance expected ({self.n}), got shape {d.shape}")
        fn = L.lib().mol_batch_step_ssprk33_f32state if f32 else L.lib().mol_batch_step_ssprk33
        L.check(fn(self._h, pu, C.c_void_p(d.ctypes.data), float(t0), int(nsteps)), batch=self._h)
        return u

    def tune(self, threads: int = 0, ctas_per_sm: int = 0, tile_cells: int = 0):
        """tile_cells > 0: tiled schedule with that tile; < 0: one CTA per instance; all 0: autotune."""
        L.check(L.lib().mol_batch_tune(self._h, int(threads), int(ctas_per_sm), int(tile_cells)), batch=self._h)

    @property
    def config(self):
        """The schedule in use: threads per CTA, CTAs per SM, tile cells (-1: one CTA per instance)."""
        th, cps, tc = C.c_int32(), C.c_int32(), C.c_int64()
        L.check(L.lib().mol_batch_config(self._h, C.byref(th), C.byref(cps), C.byref(tc)), batch=self._h)
        return {"threads": th.value, "ctas_per_sm": cps.value, "tile_cells": tc.value}

    def check(self):
        """Waits for the stream; raises if a run was abandoned after a dependency wait ran out."""
        L.check(L.lib().mol_batch_check(self._h), batch=self._h)


class ODEFunction:
    """The ODEFunction whose in-place call is the GPU RHS (src/MOL_discretization.jl:171-201)."""

    def __init__(self, plan: Plan):
        self.plan = plan

    def __call__(self, du, u, p, t):
        self.plan.rhs(du, u, p, t)
        return None


@dataclass
class ODEProblem:
    f: ODEFunction
    u0: np.ndarray
    tspan: tuple
    p: np.ndarray
    lowered: Lowered

    @property
    def plan(self) -> Plan:
        return self.f.plan


def discretize(pdesys: PDESystem, disc: MOLFiniteDifference, tspan=None) -> ODEProblem:
    """``discretize(pdesys, MOLFiniteDifference(...))`` returning a GPU-backed ODEProblem."""
    spec = pdesys.to_spec(disc)
    lw = lower(spec)
    plan = Plan(lw, expand_stencils=getattr(disc, "stencil_form", "difference") == "expanded")
    if tspan is None:
        tname = spec["time"]
        tspan = tuple(spec["domain"][tname]) if tname in spec["domain"] else (0.0, 1.0)
    u0 = lw.u0 if lw.u0 is not None else np.zeros(lw.n_unknowns)
    return ODEProblem(ODEFunction(plan), u0.copy(), tuple(tspan), lw.param_values.copy(), lw)


class SSPRK33:
    """Shu-Osher SSPRK33 (OrdinaryDiffEqSSPRK), fixed step on the device."""


class Tsit5:
    """Tsitouras 5(4) with the PI controller, adaptive on the device."""


class Solution:
    """Result of ``solve``: the final state ``u`` at time ``t`` with the integrator's ``stats``,
    and the states saved at ``ts`` (``us``).

    ``sol[u]`` (a Field, an applied field ``u(x, t)`` or a field name) gives that field on the
    full grid at every saved time, an array (len(ts), *npts) whose boundary, extrapolated,
    ghost, periodic-image and corner points are the observed values, filled in on the device
    (``mol_fill_grid``), as sol[u(t, x)] of the reference's PDETimeSeriesSolution
    (src/interface/solution/timedep.jl:19-80) holds them; ``sol[x]`` (an IV or its name) gives
    the grid's coordinates along x, and ``sol.grid`` all of them."""

    def __init__(self, u, t, stats, prob=None, ts=None, us=None):
        self.u = u
        self.t = t
        self.stats = stats
        self.prob = prob
        self.ts = np.array([t] if ts is None else ts, dtype=np.float64)
        self.us = [u] if us is None else us
        self._cache = {}

    @property
    def grid(self):
        lw = self.prob.lowered
        return {x: g.copy() for x, g in zip(lw.ivs, lw.grids)}

    def __call__(self, t, *coords, var=None):
        """Multilinear interpolation of a field over (t, x, ...) through the saved full-grid
        arrays, as the reference's ``Gridded(Linear())`` interpolation of each dependent
        variable (interface/solution/solution_utils.jl:3-32).  ``var`` names the field (a
        Field, applied field or name); it may be left out when there is only one."""
        from scipy.interpolate import RegularGridInterpolator
        lw = self.prob.lowered
        if var is None:
            if len(lw.fields) != 1:
                raise ValueError("several fields: name one with var=")
            var = lw.fields[0]
        vals = self[var]
        if len(self.ts) < 2:
            raise ValueError("interpolation in t needs at least two saved times")
        f = RegularGridInterpolator((self.ts,) + tuple(lw.grids), vals, method="linear")
        pts = np.broadcast_arrays(np.asarray(t, dtype=np.float64), *[np.asarray(c, dtype=np.float64) for c in coords])
        out = f(np.stack([p.ravel() for p in pts], axis=-1))
        return out.reshape(pts[0].shape) if pts[0].shape else float(out[0])

    def __getitem__(self, key):
        lw = self.prob.lowered
        name = key.name if isinstance(key, (IV, Field)) else (key.field.name if isinstance(key, FieldApp) else key)
        if name in lw.ivs:
            return lw.grids[lw.ivs.index(name)].copy()
        if name not in lw.fields:
            raise KeyError(name)
        if "full" not in self._cache:
            p = self.prob.p
            self._cache["full"] = np.stack([self.prob.plan.fill_grid(v, tt, p) for v, tt in zip(self.us, self.ts)])
        return self._cache["full"][:, lw.fields.index(name)]


def solve(prob: ODEProblem, alg, dt: Optional[float] = None, abstol: float = 1e-6, reltol: float = 1e-3,
          adaptive: Optional[bool] = None, u0=None, p=None, saveat=None) -> Solution:
    """Solve on the device.  ``saveat``: a step between saved times or the times themselves
    (within tspan); the start and end of tspan are saved by default.  SSPRK33 needs save
    times on its step grid; Tsit5 stops at each save time and continues from it (no
    dense-output interpolation between steps)."""
    u = np.array(prob.u0 if u0 is None else u0, dtype=np.float64, copy=True)
    t0, t1 = float(prob.tspan[0]), float(prob.tspan[1])
    p = prob.p if p is None else np.ascontiguousarray(p, dtype=np.float64)
    if saveat is None:
        marks = [t1]
    elif np.ndim(saveat) == 0:
        step = float(saveat)
        k = int(math.floor((t1 - t0) / step + 1e-9))
        marks = [t0 + i * step for i in range(1, k + 1)]
        if not marks or abs(marks[-1] - t1) > 1e-12 * max(1.0, abs(t1)):
            marks.append(t1)
    else:
        marks = sorted(float(v) for v in saveat if float(v) > t0)
    ts, us = [t0], [u.copy()]
    if isinstance(alg, SSPRK33) or alg is SSPRK33:
        if dt is None:
            raise ValueError("SSPRK33 needs dt")
        done, total = 0, 0
        for tm in marks:
            n = int(round((tm - t0) / dt))
            if abs(t0 + n * dt - tm) > 1e-9 * max(1.0, abs(tm)):
                raise ValueError(f"save time {tm} is not on the SSPRK33 step grid")
            prob.plan.step_ssprk33(u, dt, n - done, t0=t0 + done * dt, p=p)
            done = n
            ts.append(t0 + n * dt)
            us.append(u.copy())
            total = n
        return Solution(u, t0 + total * dt, {"nsteps": total}, prob, ts, us)
    if isinstance(alg, Tsit5) or alg is Tsit5:
        stats, ta = {}, t0
        agg = {"naccept": 0, "nreject": 0, "nf": 0}
        for tm in marks:
            stats = prob.plan.solve_tsit5(u, ta, tm, abstol, reltol, p=p, dt0=dt or 0.0)
            for k in agg:
                agg[k] += int(stats.get(k, 0))
            ta = stats["t"]
            ts.append(ta)
            us.append(u.copy())
        out = dict(stats)
        out.update(agg)
        return Solution(u, ta, out, prob, ts, us)
    raise ValueError(f"unsupported algorithm {alg}")
