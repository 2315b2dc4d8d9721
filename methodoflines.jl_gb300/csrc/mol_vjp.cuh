// Adjoint (vector-Jacobian product) building blocks of the discrete adjoint.
//
// Every helper is the transpose of a forward helper in mol_device.cuh: a tap
// that the forward pass *loads* is a tap the reverse pass *scatters into*
// (atomic adds, since neighbouring cells share taps).  Boundary rows are
// chained: an observed boundary value u_b = (g - b sum_k w_k u_k)/(a + b w_b)
// passes d u_b / d u_k = -b w_k / (a + b w_b) on to its interior taps.
// Gradients with respect to boundary data (a, b, g) are not propagated.
#pragma once

#include "mol_device.cuh"

namespace mol {

// Transpose of edge_row_value: d u_ghost / d u_k = -(a c_k + b d_k) / (a c_ghost + b d_ghost).
template <class T>
__device__ __noinline__ void edge_row_scatter(const DevProb<T>& P, T* lam, int f, int i0, int i1, int i2, int dout,
                                              int side, T g, T t, const T* p) {
    const int I[3] = {i0, i1, i2};
    const DevBC<T>& B = P.bc[(f * 3 + dout) * 2 + side];
    T a = B.a, b = B.b;
    if (B.prog >= 0) {
        a = run_bc_prog(P, B.prog, 0, I, t, p);
        b = run_bc_prog(P, B.prog, 1, I, t, p);
    }
    const int n = P.n[dout], pos = side == 0 ? 1 : n - 1, ghost = side == 0 ? 1 : n;
    const TapSel si = select_taps(P.ops[B.iop], pos, n, false);
    const TapSel sd = select_taps(P.ops[B.op], pos, n, false);
    T wi = T(0), wd = T(0);
    for (int k = 0; k < si.cnt; ++k)
        if (si.first + k == ghost) wi = P.w[si.woff + k];
    for (int k = 0; k < sd.cnt; ++k)
        if (sd.first + k == ghost) wd = P.w[sd.woff + k];
    const T s = -g / (a * wi + b * wd);
    int J[3] = {I[0], I[1], I[2]};
    for (int pass = 0; pass < 2; ++pass) {
        const TapSel& ts = pass == 0 ? si : sd;
        const T coef = pass == 0 ? a : b;
        for (int k = 0; k < ts.cnt; ++k) {
            const int q = ts.first + k;
            if (q == ghost) continue;
            J[dout] = q;
            bool in = true;
#pragma unroll
            for (int d = 0; d < 3; ++d) in &= (J[d] > P.lo[d]) & (J[d] <= P.n[d] - P.up[d]);
            if (in) atomicAdd(lam + (long long)f * P.ncell + flat_interior(P, J[0], J[1], J[2]), s * coef * P.w[ts.woff + k]);
        }
    }
}

template <class T>
__device__ __noinline__ void bc_row_scatter(const DevProb<T>& P, T* lam, int f, const int* I, int dout, int side,
                                            T g, T t, const T* p) {
    const DevBC<T> B = P.bc[(f * 3 + dout) * 2 + side];
#if MOL_HAS_EDGE_ROWS
    if (B.kind == MOL_BC_EDGE) {
        edge_row_scatter(P, lam, f, I[0], I[1], I[2], dout, side, g, t, p);
        return;
    }
#endif
    if (B.kind != MOL_BC_ROBIN) return;
    T a = B.a, b = B.b;
    if (B.prog >= 0) {
        a = run_bc_prog(P, B.prog, 0, I, t, p);
        b = run_bc_prog(P, B.prog, 1, I, t, p);
    }
    if (b == T(0)) return;  // Dirichlet: the boundary value does not depend on the unknowns
    const mol_op1d op = P.ops[B.op];
    const int n = P.n[dout];
    const T* w = side == 0 ? P.w + op.w_lo : P.w + op.w_hi;
    const int first = side == 0 ? 1 : n - op.bLhi + 1;
    const int cnt = side == 0 ? op.bLlo : op.bLhi;
    const int kb = side == 0 ? 0 : cnt - 1;
    const T s = B.prog >= 0 ? -b * g / (a + b * w[kb]) : -b * g * B.inv;
    int J[3] = {I[0], I[1], I[2]};
    for (int k = 0; k < cnt; ++k) {
        if (k == kb) continue;
        J[dout] = first + k;
        bool in = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) in &= (J[d] > P.lo[d]) & (J[d] <= P.n[d] - P.up[d]);
        if (in) atomicAdd(lam + (long long)f * P.ncell + flat_interior(P, J[0], J[1], J[2]), s * w[k]);
    }
}

// Transpose of bc_value: the boundary point's row, or the extrapolation row of the point
// next to it (extrap_value), whose boundary-point share goes on through the row.
template <class T>
__device__ __noinline__ void bc_scatter(const DevProb<T>& P, T* lam, int f, const int* I, int dout, int side, T g,
                                        T t, const T* p) {
    const int i = I[dout], n = P.n[dout];
    if ((side == 0 && i == 1) || (side == 1 && i == n)) {
        bc_row_scatter(P, lam, f, I, dout, side, g, t, p);
        return;
    }
    const DevBC<T>& B = P.bc[(f * 3 + dout) * 2 + side];
    if (B.xop < 0 || !((side == 0 && i == 2) || (side == 1 && i == n - 1))) return;
    const mol_op1d& x = P.ops[B.xop];
    const T* w = side == 0 ? P.w + x.w_lo + x.bLlo : P.w + x.w_hi + x.bLhi;
    const int first = side == 0 ? 1 : n - x.bLhi + 1;
    const int cnt = side == 0 ? x.bLlo : x.bLhi;
    const int qb = side == 0 ? 1 : n;
    int J[3] = {I[0], I[1], I[2]};
    for (int k = 0; k < cnt; ++k) {
        const int q = first + k;
        if (q == i) continue;
        J[dout] = q;
        if (q == qb) {
            bc_row_scatter(P, lam, f, J, dout, side, g * w[k], t, p);
            continue;
        }
        bool in = true;
#pragma unroll
        for (int d = 0; d < 3; ++d) in &= (J[d] > P.lo[d]) & (J[d] <= P.n[d] - P.up[d]);
        if (in) atomicAdd(lam + (long long)f * P.ncell + flat_interior(P, J[0], J[1], J[2]), g * w[k]);
    }
}

// Transpose of load_pt.
template <class T>
__device__ __forceinline__ void scatter_pt(const DevProb<T>& P, T* lam, int f, int i0, int i1, int i2, T g, T t,
                                           const T* p) {
    int I[3] = {i0, i1, i2};
    int nout = 0, dout = 0, side = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if ((P.permask[f] >> d) & 1) I[d] = wrap_periodic(I[d], P.n[d]);
        if (I[d] <= P.lo[d]) {
            ++nout; dout = d; side = 0;
        } else if (I[d] > P.n[d] - P.up[d]) {
            ++nout; dout = d; side = 1;
        }
    }
    if (nout == 0) {
        atomicAdd(lam + (long long)f * P.ncell + flat_interior(P, I[0], I[1], I[2]), g);
        return;
    }
    if (nout > 1) return;
    bc_scatter(P, lam, f, I, dout, side, g, t, p);
}

// Transpose of apply_op: lam[tap_k] += g w_k.
template <class T>
__device__ __noinline__ void scatter_op(const DevProb<T>& P, const mol_op1d& op, T* lam, int f, int d, const int* I,
                                        int pos, int len, T g, T t, const T* p) {
    const bool per = (P.permask[f] >> d) & 1;
    const TapSel s = select_taps(op, pos, len, per);
    int J[3] = {I[0], I[1], I[2]};
    for (int k = 0; k < s.cnt; ++k) {
        int tp = s.first + k;
        if (per) tp = wrap_periodic(tp, P.n[d]);
        J[d] = tp;
        scatter_pt(P, lam, f, J[0], J[1], J[2], g * P.w[s.woff + k], t, p);
    }
}

template <class T>
__device__ __noinline__ void scatter_mixed(const DevProb<T>& P, const mol_term& tm, T* lam, const int* I, T g, T t,
                                           const T* p) {
    const int f = tm.field, d1 = tm.dim, d2 = tm.dim2;
    const mol_op1d o1 = P.ops[tm.op], o2 = P.ops[tm.op2];
    const bool p1 = (P.permask[f] >> d1) & 1, p2 = (P.permask[f] >> d2) & 1;
    const TapSel s1 = select_taps(o1, I[d1], P.n[d1], p1);
    const TapSel s2 = select_taps(o2, I[d2], P.n[d2], p2);
    int J[3] = {I[0], I[1], I[2]};
    for (int a = 0; a < s1.cnt; ++a) {
        const T wa = P.w[s1.woff + a];
        if (wa == T(0)) continue;
        int ta = s1.first + a;
        if (s1.wrap) ta = wrap_periodic(ta, P.n[d1]);
        J[d1] = ta;
        for (int b = 0; b < s2.cnt; ++b) {
            const T wb = P.w[s2.woff + b];
            if (wb == T(0)) continue;
            int tb = s2.first + b;
            if (s2.wrap) tb = wrap_periodic(tb, P.n[d2]);
            J[d2] = tb;
            scatter_pt(P, lam, f, J[0], J[1], J[2], g * (wa * wb), t, p);
        }
    }
}

// ---------------------------------------------------------------------------
// Transposes of the line helpers of mol_device.cuh (compile-time dimension D).

template <class T, int D, bool DYN>
__device__ __noinline__ void scatter_bc_line(const DevProb<T>& P, T* lam, int f, int i0, int i1, int i2, long long c,
                                             int side, T g, T t, const T* __restrict__ p) {
    const int iD = D == 0 ? i0 : (D == 1 ? i1 : i2);
    const DevBC<T>& B = P.bc[(f * 3 + D) * 2 + side];
#if MOL_HAS_EDGE_ROWS
    if (B.kind == MOL_BC_EDGE) {
        const int e = side == 0 ? 1 : P.n[D];
        edge_row_scatter(P, lam, f, D == 0 ? e : i0, D == 1 ? e : i1, D == 2 ? e : i2, D, side, g, t, p);
        return;
    }
#endif
    if (B.kind != MOL_BC_ROBIN) return;
    if (DYN && B.prog >= 0) {
        int J[3] = {i0, i1, i2};
        J[D] = side == 0 ? 1 : P.n[D];
        bc_scatter(P, lam, f, J, D, side, g, t, p);
        return;
    }
    if (B.b == T(0)) return;
    const mol_op1d& op = P.ops[B.op];
    const int n = P.n[D];
    const T* __restrict__ w = side == 0 ? P.w + op.w_lo : P.w + op.w_hi;
    const int first = side == 0 ? 1 : n - op.bLhi + 1;
    const int cnt = side == 0 ? op.bLlo : op.bLhi;
    const int kb = side == 0 ? 0 : cnt - 1;
    const T sg = -B.b * g * B.inv;
    const long long s = gstride(P, D);
    T* lf = lam + (long long)f * P.ncell + c;
#pragma unroll 4
    for (int k = 0; k < cnt; ++k) {
        if (k == kb) continue;
        const int q = first + k;
        if (q > P.lo[D] && q <= n - P.up[D]) atomicAdd(lf + (long long)(q - iD) * s, sg * w[k]);
    }
}

// Transpose of extrap_line_value.
template <class T, int D, bool DYN>
__device__ __noinline__ void scatter_extrap_line(const DevProb<T>& P, T* lam, int f, int i0, int i1, int i2,
                                                 long long c, int side, T g, T t, const T* __restrict__ p) {
    const int iD = D == 0 ? i0 : (D == 1 ? i1 : i2);
    const DevBC<T>& B = P.bc[(f * 3 + D) * 2 + side];
    if (B.xop < 0) return;
    const mol_op1d& x = P.ops[B.xop];
    const int n = P.n[D];
    const T* __restrict__ w = side == 0 ? P.w + x.w_lo + x.bLlo : P.w + x.w_hi + x.bLhi;
    const int first = side == 0 ? 1 : n - x.bLhi + 1;
    const int cnt = side == 0 ? x.bLlo : x.bLhi;
    const int self = side == 0 ? 2 : n - 1, qb = side == 0 ? 1 : n;
    const long long s = gstride(P, D);
    T* lf = lam + (long long)f * P.ncell + c;
    for (int k = 0; k < cnt; ++k) {
        const int q = first + k;
        if (q == self) continue;
        if (q == qb) scatter_bc_line<T, D, DYN>(P, lam, f, i0, i1, i2, c, side, g * w[k], t, p);
        else if (q > P.lo[D] && q <= n - P.up[D]) atomicAdd(lf + (long long)(q - iD) * s, g * w[k]);
    }
}

// Transpose of line_edge_pt (one out-of-line call per tap).
template <class T, int D, bool DYN>
__device__ __noinline__ void scatter_line_edge_pt(const DevProb<T>& P, T* lam, int f, int i0, int i1, int i2,
                                                  long long c, int q, T g, T t, const T* __restrict__ p) {
    const int n = P.n[D];
    if (q <= P.lo[D]) {
        if (q == 1) scatter_bc_line<T, D, DYN>(P, lam, f, i0, i1, i2, c, 0, g, t, p);
#if MOL_HAS_EXTRAP_ROWS
        else if (q == 2) scatter_extrap_line<T, D, DYN>(P, lam, f, i0, i1, i2, c, 0, g, t, p);
#endif
    } else if (q == n) {
        scatter_bc_line<T, D, DYN>(P, lam, f, i0, i1, i2, c, 1, g, t, p);
    }
#if MOL_HAS_EXTRAP_ROWS
    else if (q == n - 1) {
        scatter_extrap_line<T, D, DYN>(P, lam, f, i0, i1, i2, c, 1, g, t, p);
    }
#endif
}

template <class T, int D, bool DYN>
__device__ __forceinline__ void scatter_line_pt(const DevProb<T>& P, T* lam, int f, const int* I, long long c, int q,
                                                T g, T t, const T* __restrict__ p) {
    const int n = P.n[D];
    if ((P.permask[f] >> D) & 1) q = wrap_periodic(q, n);
    if (q > P.lo[D] && q <= n - P.up[D]) {
        atomicAdd(lam + (long long)f * P.ncell + c + (long long)(q - I[D]) * gstride(P, D), g);
        return;
    }
    scatter_line_edge_pt<T, D, DYN>(P, lam, f, I[0], I[1], I[2], c, q, g, t, p);
}

template <class T, int D, int NT, bool DYN>
__device__ __forceinline__ void scatter_op_line(const DevProb<T>& P, const mol_op1d& op, T* lam, int f, const int* I,
                                                long long c, int pos, int len, T g, T t, const T* __restrict__ p) {
    const bool per = (P.permask[f] >> D) & 1;
    const TapSel s = select_taps(op, pos, len, per);
#pragma unroll
    for (int k = 0; k < NT; ++k)
        if (k < s.cnt) scatter_line_pt<T, D, DYN>(P, lam, f, I, c, s.first + k, g * P.w[s.woff + k], t, p);
}

template <class T, int D, bool DYN>
__device__ __forceinline__ void scatter_weno_taps_line(const DevProb<T>& P, int f, T* lam, const int* I, long long c,
                                                       const T* gv, T t, const T* __restrict__ p) {
#pragma unroll
    for (int k = 0; k < 5; ++k)
        scatter_line_pt<T, D, DYN>(P, lam, f, I, c, I[D] - 2 + k, gv[k], t, p);
}

// Transpose of one interior stencil line: adds v[m] to the adjoint at offset
// (OMIN + m) * s from this cell, `base` pointing at this cell's adjoint.  The share at
// offset 0 goes to `own`, which the caller adds to its cell once for all terms.  Along
// the contiguous axis (s == 1), when the 32 lanes of the warp are converged on 32
// consecutive cells, the shares that land inside the warp are summed with shuffles into
// the receiving lane's `own`; only shares leaving the warp (|offset| lanes per tap at
// each edge) are atomics.  Everything else is one atomic per nonzero share.
template <class T, int L, int OMIN, bool WARP>
__device__ __forceinline__ void scatter_taps(T* base, long long c, long long s, const T (&v)[L], T& own) {
    if (WARP && s == 1 && __activemask() == 0xffffffffu) {
        const int lane = threadIdx.x & 31;
        const long long c0 = __shfl_sync(0xffffffffu, c, 0);
        if (__all_sync(0xffffffffu, c == c0 + lane)) {
#pragma unroll
            for (int m = 0; m < L; ++m) {
                const int off = OMIN + m;
                if (off == 0) {
                    own += v[m];
                    continue;
                }
                const int src = lane - off;
                const T x = __shfl_sync(0xffffffffu, v[m], src & 31);
                if (src >= 0 && src < 32) own += x;
                const int dst = lane + off;
                if (dst < 0 || dst >= 32) atomicAdd(base + off, v[m]);
            }
            return;
        }
    }
#pragma unroll
    for (int m = 0; m < L; ++m) {
        const int off = OMIN + m;
        if (off == 0) own += v[m];
        else atomicAdd(base + (long long)off * s, v[m]);
    }
}

// scatter_taps on a periodic line: taps past either end wrap (wrap_off).  Warps with no
// wrapping lane take the shuffle path of scatter_taps.
template <class T, int L, int OMIN, bool WARP>
__device__ __forceinline__ void scatter_taps_wrap(T* base, long long c, int i, int n, long long s, const T (&v)[L],
                                                  T& own) {
    const bool wraps = i + OMIN <= 1 || i + OMIN + L - 1 > n;
    if (WARP && s == 1 && __activemask() == 0xffffffffu) {
        if (!__any_sync(0xffffffffu, wraps)) {
            scatter_taps<T, L, OMIN, true>(base, c, s, v, own);
            return;
        }
    }
#pragma unroll
    for (int m = 0; m < L; ++m) {
        const int off = OMIN + m;
        if (off == 0) own += v[m];
        else atomicAdd(base + (long long)wrap_off(i, off, n) * s, v[m]);
    }
}

// d/du_k of weno5_point: reverse mode through the same formula.  In FP64 the sweep runs
// through the one-division common-denominator form (one reciprocal of Dp*Dm serves the
// whole gradient); FP32 keeps the reciprocal form.
// Returns the point value as well (rounded differently from weno5_point: a reciprocal
// times the numerator instead of a quotient), for VJPs that need both.
template <class T>
__device__ __forceinline__ T weno5_valgrad(T um2, T um1, T u0, T up1, T up2, T eps, T inv_dx, T gr[5]) {
    const T c13_12 = T(13) / T(12);
    // products with 2 that join a sum are written as FMAs (2 x is exact: the same rounded sums)
    const T a1 = fma(T(-2), up1, u0) + up2, b1 = T(3) * u0 - T(4) * up1 + up2;
    const T a2 = fma(T(-2), u0, um1) + up1, b2 = um1 - up1;
    const T a3 = fma(T(-2), um1, um2) + u0, b3 = um2 - T(4) * um1 + T(3) * u0;
    // eps + beta_k with eps inside the FMA of the second square (0.25 b is exact)
    const T e1 = fma(c13_12 * a1, a1, fma(T(0.25) * b1, b1, eps));
    const T e2 = fma(c13_12 * a2, a2, fma(T(0.25) * b2, b2, eps));
    const T e3 = fma(c13_12 * a3, a3, fma(T(0.25) * b3, b3, eps));
    // candidate reconstructions scaled by 6 (1/6 folded into c below)
    const T hm1 = fma(T(2), up2, T(11) * u0 - T(7) * up1);
    const T hm2 = fma(T(2), um1, T(5) * u0 - up1);
    const T hm3 = T(2) * u0 + T(5) * um1 - um2;
    const T hp1 = T(2) * u0 + T(5) * up1 - up2;
    const T hp2 = T(5) * u0 + T(2) * up1 - um1;
    const T hp3 = fma(T(2), um2, T(11) * u0 - T(7) * um1);
    const T c = inv_dx * T(1.0 / 6.0);
    T gwp1, gwp2, gwp3, gwm1, gwm2, gwm3, ghp1, ghp2, ghp3, ghm1, ghm2, ghm3, ge1, ge2, ge3, val;
    if (sizeof(T) == 8) {
        const T s1 = e1 * e1, s2 = e2 * e2, s3 = e3 * e3;
        const T P1 = s2 * s3, P2 = s1 * s3, P3 = s1 * s2;
        const T wm1 = T(0.1) * P1, wm2 = T(0.6) * P2, wm3 = T(0.3) * P3;
        const T wp1 = T(0.3) * P1, wp2 = T(0.6) * P2, wp3 = T(0.1) * P3;
        const T Np = fma(wp1, hp1, fma(wp2, hp2, wp3 * hp3)), Dp = wp1 + wp2 + wp3;
        const T Nm = fma(wm1, hm1, fma(wm2, hm2, wm3 * hm3)), Dm = wm1 + wm2 + wm3;
        const T B = Dp * Dm;
        const T iB = T(1) / B;
        const T R = fma(Np, Dm, -Nm * Dp) * iB;
        val = c * R;
        // T = c * R, R = A / B, A = Np Dm - Nm Dp, B = Dp Dm
        const T gA = c * iB, gB = -c * R * iB;
        const T gNp = gA * Dm, gNm = -gA * Dp;
        const T gDp = -gA * Nm + gB * Dm, gDm = gA * Np + gB * Dp;
        gwp1 = fma(gNp, hp1, gDp); gwp2 = fma(gNp, hp2, gDp); gwp3 = fma(gNp, hp3, gDp);
        gwm1 = fma(gNm, hm1, gDm); gwm2 = fma(gNm, hm2, gDm); gwm3 = fma(gNm, hm3, gDm);
        ghp1 = gNp * wp1; ghp2 = gNp * wp2; ghp3 = gNp * wp3;
        ghm1 = gNm * wm1; ghm2 = gNm * wm2; ghm3 = gNm * wm3;
        const T gP1 = T(0.3) * gwp1 + T(0.1) * gwm1;
        const T gP2 = T(0.6) * (gwp2 + gwm2);
        const T gP3 = T(0.1) * gwp3 + T(0.3) * gwm3;
        const T gs1 = gP2 * s3 + gP3 * s2, gs2 = gP1 * s3 + gP3 * s1, gs3 = gP1 * s2 + gP2 * s1;
        ge1 = T(2) * e1 * gs1; ge2 = T(2) * e2 * gs2; ge3 = T(2) * e3 * gs3;
    } else {
        const T q1 = T(1) / (e1 * e1), q2 = T(1) / (e2 * e2), q3 = T(1) / (e3 * e3);
        const T wm1 = T(0.1) * q1, wm2 = T(0.6) * q2, wm3 = T(0.3) * q3;
        const T wp1 = T(0.3) * q1, wp2 = T(0.6) * q2, wp3 = T(0.1) * q3;
        const T Dp = wp1 + wp2 + wp3, Dm = wm1 + wm2 + wm3;
        const T hp = (wp1 * hp1 + wp2 * hp2 + wp3 * hp3) / Dp;
        const T hm = (wm1 * hm1 + wm2 * hm2 + wm3 * hm3) / Dm;
        val = (hp - hm) * c;
        const T gSp = c / Dp, gDp = -c * hp / Dp;
        const T gSm = -c / Dm, gDm = c * hm / Dm;
        gwp1 = gSp * hp1 + gDp; gwp2 = gSp * hp2 + gDp; gwp3 = gSp * hp3 + gDp;
        gwm1 = gSm * hm1 + gDm; gwm2 = gSm * hm2 + gDm; gwm3 = gSm * hm3 + gDm;
        ghp1 = gSp * wp1; ghp2 = gSp * wp2; ghp3 = gSp * wp3;
        ghm1 = gSm * wm1; ghm2 = gSm * wm2; ghm3 = gSm * wm3;
        const T gq1 = T(0.1) * gwm1 + T(0.3) * gwp1;
        const T gq2 = T(0.6) * (gwm2 + gwp2);
        const T gq3 = T(0.3) * gwm3 + T(0.1) * gwp3;
        ge1 = -T(2) * q1 / e1 * gq1; ge2 = -T(2) * q2 / e2 * gq2; ge3 = -T(2) * q3 / e3 * gq3;
    }
    // (ge 2) c13_12 = ge (2 c13_12): doubling is exact, one product fewer
    const T c13_6 = T(2) * c13_12;
    const T ga1 = ge1 * c13_6 * a1, gb1 = ge1 * T(0.5) * b1;
    const T ga2 = ge2 * c13_6 * a2, gb2 = ge2 * T(0.5) * b2;
    const T ga3 = ge3 * c13_6 * a3, gb3 = ge3 * T(0.5) * b3;
    // linear maps to (um2, um1, u0, up1, up2); the h's are unscaled here
    gr[0] = fma(T(2), ghp3, ga3 + gb3 - ghm3);
    gr[1] = fma(T(2), ghm2, fma(T(-2), ga3, ga2 + gb2) - T(4) * gb3) + T(5) * ghm3 - ghp2 - T(7) * ghp3;
    gr[2] = fma(T(2), ghp1, fma(T(2), ghm3, fma(T(-2), ga2, ga1 + T(3) * gb1) + ga3 + T(3) * gb3 + T(11) * ghm1 +
                                                T(5) * ghm2)) +
            T(5) * ghp2 + T(11) * ghp3;
    gr[3] = fma(T(2), ghp2, -T(2) * ga1 - T(4) * gb1 + ga2 - gb2 - T(7) * ghm1 - ghm2 + T(5) * ghp1);
    gr[4] = fma(T(2), ghm1, ga1 + gb1) - ghp1;
    return val;
}

template <class T>
__device__ __forceinline__ void weno5_grad(T um2, T um1, T u0, T up1, T up2, T eps, T inv_dx, T gr[5]) {
    (void)weno5_valgrad<T>(um2, um1, u0, up1, up2, eps, inv_dx, gr);
}

// Nonuniform WENO along a compile-time dimension D: the five taps of the point, its
// geometry row, and the transpose (used by the generated code).
template <class T, int D, bool DYN>
__device__ __forceinline__ T weno_nu_line(const DevProb<T>& P, const mol_term& tm, const T* __restrict__ u, int f,
                                          const int* I, long long c, T t, const T* __restrict__ p) {
    const int n = P.n[D], q0 = weno_nu_first(I[D], n);
    T v[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = line_pt<T, D, DYN>(P, u, f, I, c, q0 + k, t, p);
    const mol_op1d& o = P.ops[tm.op];
    return weno5nu_point<T>(P.w + o.w_int + (long long)(I[D] - 1) * o.L, v, T(tm.eps));
}

template <class T, int D, bool DYN>
__device__ __forceinline__ void weno_nu_line_vjp(const DevProb<T>& P, const mol_term& tm, const T* __restrict__ u,
                                                 int f, const int* I, long long c, T t, const T* __restrict__ p, T g,
                                                 T* lam) {
    const int n = P.n[D], q0 = weno_nu_first(I[D], n);
    T v[5], gr[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = line_pt<T, D, DYN>(P, u, f, I, c, q0 + k, t, p);
    const mol_op1d& o = P.ops[tm.op];
    (void)weno5nu_valgrad<T>(P.w + o.w_int + (long long)(I[D] - 1) * o.L, v, T(tm.eps), gr);
#pragma unroll
    for (int k = 0; k < 5; ++k) scatter_line_pt<T, D, DYN>(P, lam, f, I, c, q0 + k, g * gr[k], t, p);
}

// Transpose of weno_taps: gv[k] goes to tap k through the generic path.
template <class T>
__device__ __forceinline__ void scatter_weno_taps(const DevProb<T>& P, const mol_term& tm, T* lam, const int* I,
                                                  const T* gv, T t, const T* p) {
    const int f = tm.field, d = tm.dim;
    int J[3] = {I[0], I[1], I[2]};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        J[d] = I[d] - 2 + k;  // scatter_pt wraps along periodic dimensions
        scatter_pt(P, lam, f, J[0], J[1], J[2], gv[k], t, p);
    }
}

template <class T>
__device__ __noinline__ void scatter_weno(const DevProb<T>& P, const mol_term& tm, const T* u, T* lam, const int* I, T g,
                                          T t, const T* p) {
    T v[5];
    if (tm.variant == 1) {  // nonuniform: taps q0..q0+4, geometry row of the point
        const int d = tm.dim, n = P.n[d], q0 = weno_nu_first(I[d], n);
        int J[3] = {I[0], I[1], I[2]};
        for (int k = 0; k < 5; ++k) {
            J[d] = q0 + k;
            v[k] = load_pt(P, u, tm.field, J[0], J[1], J[2], t, p);
        }
        const mol_op1d& o = P.ops[tm.op];
        T gr[5];
        (void)weno5nu_valgrad<T>(P.w + o.w_int + (long long)(I[d] - 1) * o.L, v, T(tm.eps), gr);
        for (int k = 0; k < 5; ++k) {
            J[d] = q0 + k;
            scatter_pt(P, lam, tm.field, J[0], J[1], J[2], g * gr[k], t, p);
        }
        return;
    }
    weno_taps(P, tm, u, I, t, p, v);
    T gr[5];
    weno5_grad<T>(v[0], v[1], v[2], v[3], v[4], T(tm.eps), T(tm.dx), gr);
#pragma unroll
    for (int k = 0; k < 5; ++k) gr[k] *= g;
    scatter_weno_taps(P, tm, lam, I, gr, t, p);
}

}  // namespace mol
