"""Slab decomposition of one problem over several GPUs, one process per GPU.

The unknowns are split along the slowest spatial dimension into contiguous slabs of planes,
one slab per rank.  Each rank holds its slab plus `halo` ghost planes on either side, and its
local problem is the global one with that dimension replaced by a periodic dimension of
(slab + 2 halo) planes.  Every stencil reaches at most `halo` planes, so once the ghost planes
hold the neighbours' planes the local right-hand side at every owned plane is the global one:
the wrap only ever joins ghost planes to ghost planes, and what the local problem computes at
ghost planes is overwritten by the next exchange.  Ghost planes are refreshed before every
right-hand side evaluation with one point-to-point exchange per neighbour
(torch.distributed send/recv: NCCL between GPUs, gloo between CPU processes); the batched
ensemble needs none of this and shards by instance.

Where the global dimension is bounded, its boundary rows must be constant Dirichlet rows and
every stencil along it must reach one plane: the end rank's ghost plane then holds the
boundary value, which is what the boundary row makes the stencil read.  Arrays the lowering
hoisted out of the right-hand side (coefficients at cells, faces and boundary points) are
cut out of the global arrays, so the local plans use the global values.
"""
from __future__ import annotations

import copy
from typing import Callable, List, Optional

import numpy as np

from . import _lib as L
from .lowering import Lowered


def _prog_aux(lw: Lowered, prog: int) -> List[int]:
    """aux indices read (MOL_OP_AUX) by a program."""
    if prog is None or prog < 0:
        return []
    return [imm for (op, dst, a, b, c, imm) in lw.programs[prog] if op == L.OP_AUX]


def _reach(o) -> int:
    return max(abs(o.omin), abs(o.omin + o.L - 1))


class Slab:
    """Rank `rank` of `world`'s part of the lowered problem `lw`: `local` is the lowered local
    problem (make a Plan of it), `p0:p1` the owned planes of the slowest dimension."""

    def __init__(self, lw: Lowered, rank: int, world: int, halo: Optional[int] = None):
        self.lw, self.rank, self.world = lw, rank, world
        nd = len(lw.ivs)
        D = nd - 1
        self.D = D
        nf = len(lw.fields)
        per = [lw.periodic[f][D] for f in lw.fields]
        if len(set(per)) != 1:
            raise NotImplementedError("slabs: every field must be periodic along the slowest dimension, or none")
        self.periodic = per[0]
        if not lw.uniform[D]:
            raise NotImplementedError("slabs: the slowest dimension must be uniform")
        # reach of the stencils along D (nonlinear Laplacian: outer face plus its inner and
        # interpolation stencils)
        reach = 0
        for t in lw.terms:
            dims = [t["dim"]] + ([t["dim2"]] if t["kind"] == L.TERM_MIXED else [])
            if D not in dims:
                continue
            if t["kind"] == L.TERM_WENO:
                reach = max(reach, 2)
            elif t["kind"] == L.TERM_NONLINLAP:
                # faces at II + r (r from the outer stencil, which sits at II - 1), each reading
                # the inner derivative's taps and, when the coefficient depends on a field, the
                # interpolation's taps around it
                oo, oi, op = lw.ops[t["op"]], lw.ops[t["op2"]], lw.ops[t["op3"]]
                prog = lw.programs[t["prog"]] if t.get("prog", -1) >= 0 else []
                taps = [oi] + ([op] if any(ins[0] == L.OP_FIELD for ins in prog) else [])
                for m in range(oo.L):
                    r = oo.omin + m - 1
                    for o in taps:
                        for q in range(o.L):
                            reach = max(reach, abs(r + o.omin + q))
            else:
                op = t["op"] if t["dim"] == D else t["op2"]
                reach = max(reach, _reach(lw.ops[op]))
        h = max(1, reach) if halo is None else int(halo)
        if h < reach:
            raise ValueError(f"slabs: halo {h} is below the stencils' reach {reach}")
        self.fill = [0.0] * nf
        if not self.periodic:
            if h != 1 or reach > 1:
                raise NotImplementedError("slabs: a bounded slowest dimension needs stencils that reach one plane")
            for f in range(nf):
                for side in (0, 1):
                    e = lw.bcs.get((f, D, side))
                    if e is None or e["kind"] != L.BC_ROBIN or e["prog"] >= 0 or e["b"] != 0.0 or e.get("extrap", 0):
                        raise NotImplementedError("slabs: a bounded slowest dimension needs constant Dirichlet rows")
                    v = e["g"] / e["a"]
                    if side == 0:
                        self.fill[f] = v
                    elif v != self.fill[f]:
                        raise NotImplementedError("slabs: different Dirichlet values at the two ends")
            if lw.lower[D] != 1 or lw.upper[D] != 1:
                raise NotImplementedError("slabs: one boundary point at each end of the slowest dimension")
        self.h = h
        N = lw.npts[D] - lw.lower[D] - lw.upper[D]
        self.N = N
        b = [N * r // world for r in range(world + 1)]
        self.bounds = b
        self.p0, self.p1 = b[rank], b[rank + 1]
        self.nloc = self.p1 - self.p0
        if min(b[r + 1] - b[r] for r in range(world)) < h:
            raise ValueError(f"slabs: {world} slabs of {N} planes leave a slab thinner than the halo {h}")
        self.Lp = self.nloc + 2 * h                       # local unknown planes (ghosts included)
        self.plane = int(np.prod(lw.interior_shape[:D])) if D > 0 else 1
        self.local = self._local_problem()

    # ------------------------------------------------------------------ geometry
    def _point(self, p: int) -> int:
        """0-based global grid point of global unknown plane p (wrapped when periodic), or -1
        beyond a bounded end (p = -1 and p = N are the boundary points themselves)."""
        lw, D = self.lw, self.D
        if self.periodic:
            return lw.lower[D] + (p % self.N)
        q = lw.lower[D] + p
        return q if 0 <= q < lw.npts[D] else -1

    def _local_planes(self):
        """Global unknown plane of each local plane 0..Lp-1."""
        return [self.p0 - self.h + k for k in range(self.Lp)]

    def _local_problem(self) -> Lowered:
        lw, D = self.lw, self.D
        loc = copy.copy(lw)
        planes = self._local_planes()
        pts = [self._point(p) for p in planes]
        # grid along D: the wrap image (point 1) then the local planes; the image sits one step
        # before the first local plane (only the ghost planes' discarded values can see it)
        g = lw.grids[D]
        dx = lw.dx[D]
        coords = [g[q] if q >= 0 else g[0] + (p + lw.lower[D]) * dx for p, q in zip(planes, pts)]
        loc.grids = list(lw.grids)
        loc.grids[D] = np.array([coords[0] - dx] + coords, dtype=np.float64)
        loc.npts = list(lw.npts)
        loc.npts[D] = self.Lp + 1
        loc.lower = list(lw.lower)
        loc.upper = list(lw.upper)
        loc.lower[D], loc.upper[D] = 1, 0
        loc.periodic = {f: list(v) for f, v in lw.periodic.items()}
        for f in loc.periodic:
            loc.periodic[f][D] = True
        loc.bcs = {k: v for k, v in lw.bcs.items() if k[1] != D}
        for fi in range(len(lw.fields)):
            loc.bcs[(fi, D, 0)] = {"kind": L.BC_PERIODIC, "op": 0, "prog": -1, "a": 0.0, "b": 0.0, "g": 0.0}
        # hoisted arrays: classify by their readers, cut along D
        kind = {}
        for k in _prog_aux(lw, lw.cell_prog):
            kind[k] = ("cell", None)
        for t in lw.terms:
            if t["kind"] == L.TERM_NONLINLAP:
                for k in _prog_aux(lw, t["prog"]):
                    kind[t["aux0"] + k] = ("face", t["dim"])
        for e in lw.bcs.values():
            for k in _prog_aux(lw, e.get("prog", -1)):
                kind.setdefault(k, ("grid", None))
        aux = []
        for k, a in enumerate(lw.aux):
            kd, fdim = kind.get(k, ("cell", None))
            aux.append(self._cut(a, kd, fdim, planes, pts))
        loc.aux = aux
        loc.u0 = self.scatter(lw.u0, fill_ghosts=True)
        return loc

    def _cut(self, a: np.ndarray, kd: str, fdim, planes, pts) -> np.ndarray:
        lw, D = self.lw, self.D
        nd = len(lw.ivs)
        if kd == "cell":
            shp = list(lw.interior_shape)
            arr = a.reshape(shp, order="F")
            idx = [p % self.N if self.periodic else p for p in planes]
            ok = [0 <= p < self.N for p in idx]
            out = np.zeros(shp[:D] + [self.Lp], dtype=np.float64)
            for k, (p, good) in enumerate(zip(idx, ok)):
                if good:
                    out[..., k] = arr[..., p]
            return np.ascontiguousarray(out.reshape(-1, order="F"))
        ext = [lw.npts[d] + (1 if (kd == "face" and fdim == d) else 0) for d in range(nd)]
        arr = a.reshape(ext, order="F")
        if kd == "face" and fdim == D:
            # local half point Ih (between local points Ih and Ih + 1, 1-based) -> the global
            # half point after the global point of local point Ih
            lpts = [self._point(self.p0 - self.h - 1)] + pts     # local points 1 .. Lp + 1
            n_out = self.Lp + 2
            out = np.zeros(ext[:D] + [n_out], dtype=np.float64)
            for Ih in range(1, self.Lp + 2):
                q = lpts[Ih - 1] if Ih - 1 < len(lpts) else -1
                if q >= 0:
                    out[..., Ih] = arr[..., q + 1]
            return np.ascontiguousarray(out.reshape(-1, order="F"))
        lpts = [self._point(self.p0 - self.h - 1)] + pts
        out = np.zeros(ext[:D] + [self.Lp + 1], dtype=np.float64)
        for k, q in enumerate(lpts):
            if q >= 0:
                out[..., k] = arr[..., q]
        return np.ascontiguousarray(out.reshape(-1, order="F"))

    # ------------------------------------------------------------------ state maps
    def scatter(self, u_global: np.ndarray, fill_ghosts: bool = True) -> np.ndarray:
        """This rank's local state (owned planes and, with fill_ghosts, the ghost planes) cut
        out of a global state vector."""
        nf, S, N = len(self.lw.fields), self.plane, self.N
        g = np.asarray(u_global).reshape(nf, N, S)
        out = np.zeros((nf, self.Lp, S), dtype=np.float64)
        for k, p in enumerate(self._local_planes()):
            q = p % N if self.periodic else p
            if 0 <= q < N:
                out[:, k, :] = g[:, q, :]
            elif fill_ghosts:
                out[:, k, :] = np.array(self.fill)[:, None]
        return out.reshape(-1)

    def owned(self, u_local):
        """The owned planes of a local state, (fields, planes, plane cells)."""
        nf, S = len(self.lw.fields), self.plane
        return u_local.reshape(nf, self.Lp, S)[:, self.h:self.h + self.nloc, :]

    # ------------------------------------------------------------------ halo exchange
    def exchange(self, u_local, dist=None):
        """Fill the ghost planes of the local state `u_local` (a torch tensor) from the
        neighbouring ranks' owned planes (torch.distributed point-to-point), or with the
        boundary value at a bounded end.  One message per neighbour."""
        import torch
        nf, S, h, n = len(self.lw.fields), self.plane, self.h, self.nloc
        v = u_local.view(nf, self.Lp, S)
        lo_nb = self.rank - 1 if (self.rank > 0 or self.periodic) else None
        hi_nb = self.rank + 1 if (self.rank < self.world - 1 or self.periodic) else None
        if lo_nb is not None:
            lo_nb %= self.world
        if hi_nb is not None:
            hi_nb %= self.world
        send_lo = v[:, h:2 * h, :].contiguous()          # -> the lower neighbour's high ghosts
        send_hi = v[:, n:n + h, :].contiguous()          # -> the upper neighbour's low ghosts
        recv_lo = torch.empty_like(send_lo)
        recv_hi = torch.empty_like(send_hi)
        if self.world == 1:
            if self.periodic:
                recv_lo.copy_(send_hi)
                recv_hi.copy_(send_lo)
        else:
            dist = dist or torch.distributed
            # sends upward then downward, receives from below then from above: with two ranks
            # on a periodic dimension both neighbours are one rank, and messages between one
            # pair are matched in issue order (NCCL has no tags; gloo gets them too)
            ops = []
            if hi_nb is not None:
                ops.append(dist.P2POp(dist.isend, send_hi, hi_nb, tag=1))
            if lo_nb is not None:
                ops.append(dist.P2POp(dist.isend, send_lo, lo_nb, tag=2))
            if lo_nb is not None:
                ops.append(dist.P2POp(dist.irecv, recv_lo, lo_nb, tag=1))
            if hi_nb is not None:
                ops.append(dist.P2POp(dist.irecv, recv_hi, hi_nb, tag=2))
            for r in dist.batch_isend_irecv(ops):
                r.wait()
        if lo_nb is not None:
            v[:, 0:h, :] = recv_lo
        else:
            for f in range(nf):
                v[f, 0:h, :] = self.fill[f]
        if hi_nb is not None:
            v[:, n + h:n + 2 * h, :] = recv_hi
        else:
            for f in range(nf):
                v[f, n + h:n + 2 * h, :] = self.fill[f]

    # ------------------------------------------------------------------ stepping
    @staticmethod
    def exchange_in_process(slabs: List["Slab"], states) -> None:
        """The exchange of every slab of one decomposition held by one process (one state
        tensor per slab, in rank order, on one or several devices): the same ghost planes as
        `exchange`, filled by tensor copies."""
        world = len(slabs)
        for r, sl in enumerate(slabs):
            nf, h, n = len(sl.lw.fields), sl.h, sl.nloc
            v = states[r].view(nf, sl.Lp, sl.plane)
            lo = (r - 1) % world if (r > 0 or sl.periodic) else None
            hi = (r + 1) % world if (r < world - 1 or sl.periodic) else None
            if lo is not None:
                s2 = slabs[lo]
                v[:, 0:h, :] = states[lo].view(nf, s2.Lp, s2.plane)[:, s2.nloc:s2.nloc + h, :].to(v.device)
            else:
                for f in range(nf):
                    v[f, 0:h, :] = sl.fill[f]
            if hi is not None:
                s2 = slabs[hi]
                v[:, n + h:n + 2 * h, :] = states[hi].view(nf, s2.Lp, s2.plane)[:, h:2 * h, :].to(v.device)
            else:
                for f in range(nf):
                    v[f, n + h:n + 2 * h, :] = sl.fill[f]

    def ssprk33(self, u, dt: float, nsteps: int, rhs: Callable, t0: float = 0.0, exchange: Callable = None):
        """nsteps SSPRK33 steps of the local state `u` (a torch tensor, in place) with
        OrdinaryDiffEq's stage order; `rhs(du, u, t)` evaluates the local right-hand side
        (Plan.rhs on a GPU); the ghost planes are exchanged before every evaluation."""
        import torch
        ex = exchange or self.exchange
        k = torch.empty_like(u)
        t = t0
        for _ in range(nsteps):
            ex(u)
            rhs(k, u, t)
            u1 = u + dt * k
            ex(u1)
            rhs(k, u1, t + dt)
            u2 = ((3.0 * u + u1) + dt * k) * 0.25
            ex(u2)
            rhs(k, u2, t + dt / 2)
            u.copy_(((u + 2.0 * u2) + (2.0 * dt) * k) / 3.0)
            t = t + dt
        return u
