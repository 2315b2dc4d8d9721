"""CPU model of the descriptor semantics the CUDA kernels implement (test helper).

Evaluates f(du, u, p, t) straight from a lowered descriptor, one cell at a
time, with the same tap selection, boundary-row resolution and register
program as ``mol_device.cuh``.  Comparing it with the oracle checks the host
lowering on machines without a GPU; comparing the GPU with the oracle checks
the kernels.
"""
from __future__ import annotations

import math

import numpy as np

from molgpu import _lib as L
from molgpu.weights import select, wrap


class DescInterp:
    def __init__(self, lw):
        self.lw = lw
        self.nd = len(lw.ivs)
        self.n = list(lw.npts) + [1] * (3 - self.nd)
        self.lo = list(lw.lower) + [0] * (3 - self.nd)
        self.up = list(lw.upper) + [0] * (3 - self.nd)
        self.ni = [self.n[d] - self.lo[d] - self.up[d] for d in range(3)]
        self.ncell = int(np.prod(self.ni))
        self.per = {fi: [lw.periodic[f][d] if d < self.nd else False for d in range(3)]
                    for fi, f in enumerate(lw.fields)}

    def flat(self, I):
        return (I[0] - 1 - self.lo[0]) + self.ni[0] * ((I[1] - 1 - self.lo[1]) + self.ni[1] * (I[2] - 1 - self.lo[2]))

    def load(self, u, f, I, t, p):
        I = list(I)
        out = []
        for d in range(3):
            if self.per[f][d]:
                I[d] = wrap(I[d], self.n[d])
            if I[d] <= self.lo[d]:
                out.append((d, 0))
            elif I[d] > self.n[d] - self.up[d]:
                out.append((d, 1))
        if not out:
            return u[f * self.ncell + self.flat(I)]
        if len(out) > 1:
            return 0.0
        d, side = out[0]
        e = self.lw.bcs.get((f, d, side))
        nxt = 2 if side == 0 else self.n[d] - 1
        if e is not None and e.get("extrap", 0) and I[d] == nxt:
            # extrapolated point next to the boundary point (extrap_value)
            xo = self.lw.ops[e["extrap"] - 1]
            w = xo.low[1] if side == 0 else xo.high[1]
            first = 1 if side == 0 else self.n[d] - xo.bLhi + 1
            acc = None
            for k, wk in enumerate(w):
                q = first + k
                if q == I[d]:
                    continue
                J = list(I)
                J[d] = q
                term = wk * self.load(u, f, J, t, p)
                acc = term if acc is None else acc + term
            return acc
        if (side == 0 and I[d] != 1) or (side == 1 and I[d] != self.n[d]):
            return 0.0
        if e is None or e["kind"] not in (L.BC_ROBIN, L.BC_EDGE):
            return 0.0
        a, b, g = e["a"], e["b"], e["g"]
        if e["prog"] >= 0:
            a, b, g = self.run_prog(e["prog"], "bc", None, I, t, p, u)
        if e["kind"] == L.BC_EDGE:
            # edge_row_value: interpolation and half-offset derivative at the face
            pos, ghost = (1, 1) if side == 0 else (self.n[d] - 1, self.n[d])
            sums, cg = [], []
            for opi in (e["iop"], e["op"]):
                w, taps = select(self.lw.ops[opi], pos, self.n[d], False)
                acc, c = 0.0, 0.0
                for wk, q in zip(w, taps):
                    if q == ghost:
                        c = wk
                        continue
                    J = list(I)
                    J[d] = q
                    acc = acc + wk * u[f * self.ncell + self.flat(J)]
                sums.append(acc)
                cg.append(c)
            return (g - a * sums[0] - b * sums[1]) / (a * cg[0] + b * cg[1])
        if b == 0.0:
            return g / a
        op = self.lw.ops[e["op"]]
        w = op.low[0] if side == 0 else op.high[0]
        first = 1 if side == 0 else self.n[d] - op.bLhi + 1
        kb = 0 if side == 0 else len(w) - 1
        acc = None
        for k in range(len(w)):
            if k == kb:
                continue
            J = list(I)
            J[d] = first + k
            inside = all(self.lo[q] < J[q] <= self.n[q] - self.up[q] for q in range(3))
            v = u[f * self.ncell + self.flat(J)] if inside else 0.0
            term = w[k] * v
            acc = term if acc is None else acc + term
        return (g - b * acc) / (a + b * w[kb])

    def apply_op(self, op, u, f, d, I, t, p, length=None, pos=None):
        per = self.per[f][d]
        n = self.n[d]
        i = I[d] if pos is None else pos
        w, taps = select(op, i, n if length is None else length, per)
        acc = 0.0
        for k, (wk, tk) in enumerate(zip(w, taps)):
            if per:
                tk = wrap(tk, n)
            J = list(I)
            J[d] = tk
            v = self.load(u, f, J, t, p)
            acc = wk * v if k == 0 else acc + wk * v
        return acc

    def term(self, k, u, I, t, p):
        tm = self.lw.terms[k]
        kind = tm["kind"]
        f = tm["field"]
        d = tm["dim"]
        if kind == L.TERM_LINEAR:
            return self.apply_op(self.lw.ops[tm["op"]], u, f, d, I, t, p)
        if kind == L.TERM_MIXED:
            d2 = tm["dim2"]
            o1, o2 = self.lw.ops[tm["op"]], self.lw.ops[tm["op2"]]
            w1, t1 = select(o1, I[d], self.n[d], self.per[f][d])
            w2, t2 = select(o2, I[d2], self.n[d2], self.per[f][d2])
            acc = 0.0
            for wa, ta in zip(w1, t1):
                for wb, tb in zip(w2, t2):
                    J = list(I)
                    J[d] = wrap(ta, self.n[d]) if self.per[f][d] else ta
                    J[d2] = wrap(tb, self.n[d2]) if self.per[f][d2] else tb
                    acc += wa * wb * self.load(u, f, J, t, p)
            return acc
        if kind == L.TERM_WENO:
            if tm.get("variant", 0) == 1:
                from molgpu.weights import weno_nonuniform_target
                q0, _ = weno_nonuniform_target(I[d], self.n[d])
                v = []
                for k in range(5):
                    J = list(I)
                    J[d] = q0 + k
                    v.append(self.load(u, f, J, t, p))
                return _weno_nu(self.lw.ops[tm["op"]].rows[I[d] - 1], v, tm["eps"])
            v = []
            for o in range(-2, 3):
                J = list(I)
                J[d] = I[d] + o  # load wraps along periodic dimensions
                v.append(self.load(u, f, J, t, p))
            return _weno(*v, tm["eps"], tm["dx"])
        if kind == L.TERM_NONLINLAP:
            n = self.n[d]
            per = self.per[f][d]
            oo = self.lw.ops[tm["op"]]
            wo, to = select(oo, I[d] - 1, n - 1, per)
            acc = 0.0
            for w_, Ih in zip(wo, to):
                if w_ == 0.0:
                    continue
                du = self.apply_op(self.lw.ops[tm["op2"]], u, f, d, I, t, p, pos=Ih)
                a = 1.0
                if tm.get("prog", -1) >= 0:
                    a = self.run_prog(tm["prog"], "face", (tm, Ih), I, t, p, u)
                acc += w_ * (a * du)
            return acc
        raise ValueError(kind)

    def run_prog(self, prog, kind, face, I, t, p, u, c=None):
        r = {}
        outs = {}
        for (op, dst, a, b, cc, imm) in self.lw.programs[prog]:
            if op == L.OP_CONST:
                r[dst] = self.lw.consts[imm]
            elif op == L.OP_PARAM:
                r[dst] = p[imm]
            elif op == L.OP_FIELD:
                if kind == "face":
                    tm, Ih = face
                    r[dst] = self.apply_op(self.lw.ops[tm["op3"]], u, imm, tm["dim"], I, t, p, pos=Ih)
                else:
                    r[dst] = u[imm * self.ncell + c]
            elif op == L.OP_AUX:
                if kind == "face":
                    tm, Ih = face
                    d = tm["dim"]
                    e0 = self.n[0] + (d == 0)
                    e1 = self.n[1] + (d == 1)
                    j = [Ih if q == d else I[q] - 1 for q in range(3)]
                    r[dst] = self.lw.aux[tm["aux0"] + imm][j[0] + e0 * (j[1] + e1 * j[2])]
                elif kind == "bc":   # full-grid array, read at the boundary point
                    r[dst] = self.lw.aux[imm][(I[0] - 1) + self.n[0] * ((I[1] - 1) + self.n[1] * (I[2] - 1))]
                else:
                    r[dst] = self.lw.aux[imm][c]
            elif op == L.OP_COORD:
                r[dst] = self.lw.grids[imm][I[imm] - 1]
            elif op == L.OP_TIME:
                r[dst] = t
            elif op == L.OP_TERM:
                r[dst] = self.term(imm, u, I, t, p)
            elif op == L.OP_UPWIND:
                kap = r[a]
                r[dst] = kap * self.term(b, u, I, t, p) if kap < 0 else kap * self.term(cc, u, I, t, p)
            elif op == L.OP_ADD:
                r[dst] = r[a] + r[b]
            elif op == L.OP_SUB:
                r[dst] = r[a] - r[b]
            elif op == L.OP_MUL:
                r[dst] = r[a] * r[b]
            elif op == L.OP_DIV:
                r[dst] = r[a] / r[b]
            elif op == L.OP_NEG:
                r[dst] = -r[a]
            elif op == L.OP_POWI:
                x = r[a]
                r[dst] = x * x if imm == 2 else (x * x * x if imm == 3 else x ** imm)
            elif op == L.OP_POW:
                r[dst] = r[a] ** r[b]
            elif op == L.OP_FN:
                name = [k for k, v in L.FN_IDS.items() if v == imm][0]
                r[dst] = abs(r[a]) if name == "abs" else getattr(math, name)(r[a])
            elif op == L.OP_CMP:
                x, y = r[a], r[b]
                r[dst] = float({0: x <= y, 1: x < y, 2: x >= y, 3: x > y, 4: x == y}[imm])
            elif op == L.OP_IFELSE:
                r[dst] = r[b] if r[a] != 0 else r[cc]
            elif op == L.OP_OUT:
                outs[imm] = r[a]
        if kind == "bc":
            return outs.get(0, 0.0), outs.get(1, 0.0), outs.get(2, 0.0)
        if kind == "face":
            return outs[0]
        return outs

    def rhs(self, u, t, p=None):
        p = self.lw.param_values if p is None else p
        du = np.zeros(self.ncell * len(self.lw.fields))
        for c in range(self.ncell):
            c0 = c % self.ni[0]
            r = c // self.ni[0]
            I = [c0 + 1 + self.lo[0], r % self.ni[1] + 1 + self.lo[1], r // self.ni[1] + 1 + self.lo[2]]
            outs = self.run_prog(self.lw.cell_prog, "cell", None, I, t, p, u, c)
            for f, v in outs.items():
                du[f * self.ncell + c] = v
        return du


def _weno(um2, um1, u0, up1, up2, eps, dx):
    b1 = 13 * (u0 - 2 * up1 + up2) ** 2 / 12 + (3 * u0 - 4 * up1 + up2) ** 2 / 4
    b2 = 13 * (um1 - 2 * u0 + up1) ** 2 / 12 + (um1 - up1) ** 2 / 4
    b3 = 13 * (um2 - 2 * um1 + u0) ** 2 / 12 + (um2 - 4 * um1 + 3 * u0) ** 2 / 4
    q = [1 / (eps + b) ** 2 for b in (b1, b2, b3)]
    wm = [0.1 * q[0], 0.6 * q[1], 0.3 * q[2]]
    wp = [0.3 * q[0], 0.6 * q[1], 0.1 * q[2]]
    hm = [(11 * u0 - 7 * up1 + 2 * up2) / 6, (5 * u0 - up1 + 2 * um1) / 6, (2 * u0 + 5 * um1 - um2) / 6]
    hp = [(2 * u0 + 5 * up1 - up2) / 6, (5 * u0 + 2 * up1 - um1) / 6, (11 * u0 - 7 * um1 + 2 * um2) / 6]
    return (sum(a * b for a, b in zip(wp, hp)) / sum(wp) - sum(a * b for a, b in zip(wm, hm)) / sum(wm)) / dx


def _weno_nu(g, v, eps):
    """weno5nu_point: the nonuniform WENO from a point's geometry row."""
    b, r = [], []
    for k in range(3):
        m = g[3 + 15 * k:3 + 15 * (k + 1)]
        a = v[k:k + 3]

        def d3(w):
            return w[0] * a[0] + w[1] * a[1] + w[2] * a[2]
        rr, pL, pM, pR, pp = d3(m[0:3]), d3(m[3:6]), d3(m[6:9]), d3(m[9:12]), d3(m[12:15])
        val = g[1] * (g[0] * (pL * pL + 4 * (pM * pM) + pR * pR)) + g[2] * (g[1] * (pp * pp))
        b.append(max(val, 0.0))
        r.append(rr)
    ap = [g[48 + k] / ((eps + b[k]) * (eps + b[k])) for k in range(3)]
    am = [g[51 + k] / ((eps + b[k]) * (eps + b[k])) for k in range(3)]
    sp, sm = ap[0] + ap[1] + ap[2], am[0] + am[1] + am[2]
    Rp = (ap[0] / sp) * r[0] + (ap[1] / sp) * r[1] + (ap[2] / sp) * r[2]
    Rm = (am[0] / sm) * r[0] + (am[1] / sm) * r[1] + (am[2] / sm) * r[2]
    return g[54] * Rp - g[55] * Rm
