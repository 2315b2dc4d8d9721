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

template <class T>
__device__ __noinline__ void bc_scatter(const DevProb<T>& P, T* lam, int f, const int* I, int dout, int side, T g,
                                        T t, const T* p) {
    if ((side == 0 && I[dout] != 1) || (side == 1 && I[dout] != P.n[dout])) return;
    const DevBC<T> B = P.bc[(f * 3 + dout) * 2 + side];
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
    const T s = -b * g / (a + b * w[kb]);
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

// d/du_k of weno5_point (reverse mode through the same formula).
template <class T>
__device__ __forceinline__ void weno5_grad(T um2, T um1, T u0, T up1, T up2, T eps, T inv_dx, T gr[5]) {
    const T c13_12 = T(13) / T(12);
    const T a1 = u0 - T(2) * up1 + up2, b1 = T(3) * u0 - T(4) * up1 + up2;
    const T a2 = um1 - T(2) * u0 + up1, b2 = um1 - up1;
    const T a3 = um2 - T(2) * um1 + u0, b3 = um2 - T(4) * um1 + T(3) * u0;
    const T e1 = eps + fma(c13_12 * a1, a1, T(0.25) * (b1 * b1));
    const T e2 = eps + fma(c13_12 * a2, a2, T(0.25) * (b2 * b2));
    const T e3 = eps + fma(c13_12 * a3, a3, T(0.25) * (b3 * b3));
    const T q1 = T(1) / (e1 * e1), q2 = T(1) / (e2 * e2), q3 = T(1) / (e3 * e3);
    const T wm1 = T(0.1) * q1, wm2 = T(0.6) * q2, wm3 = T(0.3) * q3;
    const T wp1 = T(0.3) * q1, wp2 = T(0.6) * q2, wp3 = T(0.1) * q3;
    const T sixth = T(1) / T(6);
    const T hm1 = (T(11) * u0 - T(7) * up1 + T(2) * up2) * sixth;
    const T hm2 = (T(5) * u0 - up1 + T(2) * um1) * sixth;
    const T hm3 = (T(2) * u0 + T(5) * um1 - um2) * sixth;
    const T hp1 = (T(2) * u0 + T(5) * up1 - up2) * sixth;
    const T hp2 = (T(5) * u0 + T(2) * up1 - um1) * sixth;
    const T hp3 = (T(11) * u0 - T(7) * um1 + T(2) * um2) * sixth;
    const T Dp = wp1 + wp2 + wp3, Dm = wm1 + wm2 + wm3;
    const T hp = (wp1 * hp1 + wp2 * hp2 + wp3 * hp3) / Dp;
    const T hm = (wm1 * hm1 + wm2 * hm2 + wm3 * hm3) / Dm;
    // reverse
    const T gSp = inv_dx / Dp, gDp = -inv_dx * hp / Dp;
    const T gSm = -inv_dx / Dm, gDm = inv_dx * hm / Dm;
    const T gwp1 = gSp * hp1 + gDp, gwp2 = gSp * hp2 + gDp, gwp3 = gSp * hp3 + gDp;
    const T gwm1 = gSm * hm1 + gDm, gwm2 = gSm * hm2 + gDm, gwm3 = gSm * hm3 + gDm;
    const T ghp1 = gSp * wp1, ghp2 = gSp * wp2, ghp3 = gSp * wp3;
    const T ghm1 = gSm * wm1, ghm2 = gSm * wm2, ghm3 = gSm * wm3;
    const T gq1 = T(0.1) * gwm1 + T(0.3) * gwp1;
    const T gq2 = T(0.6) * (gwm2 + gwp2);
    const T gq3 = T(0.3) * gwm3 + T(0.1) * gwp3;
    const T ge1 = -T(2) * q1 / e1 * gq1, ge2 = -T(2) * q2 / e2 * gq2, ge3 = -T(2) * q3 / e3 * gq3;
    const T ga1 = ge1 * T(2) * c13_12 * a1, gb1 = ge1 * T(0.5) * b1;
    const T ga2 = ge2 * T(2) * c13_12 * a2, gb2 = ge2 * T(0.5) * b2;
    const T ga3 = ge3 * T(2) * c13_12 * a3, gb3 = ge3 * T(0.5) * b3;
    // linear maps to (um2, um1, u0, up1, up2)
    T g_um2 = ga3 + gb3 - ghm3 * sixth + T(2) * ghp3 * sixth;
    T g_um1 = ga2 + gb2 - T(2) * ga3 - T(4) * gb3 + T(2) * ghm2 * sixth + T(5) * ghm3 * sixth - ghp2 * sixth -
              T(7) * ghp3 * sixth;
    T g_u0 = ga1 + T(3) * gb1 - T(2) * ga2 + ga3 + T(3) * gb3 +
             (T(11) * ghm1 + T(5) * ghm2 + T(2) * ghm3 + T(2) * ghp1 + T(5) * ghp2 + T(11) * ghp3) * sixth;
    T g_up1 = -T(2) * ga1 - T(4) * gb1 + ga2 - gb2 + (-T(7) * ghm1 - ghm2 + T(5) * ghp1 + T(2) * ghp2) * sixth;
    T g_up2 = ga1 + gb1 + (T(2) * ghm1 - ghp1) * sixth;
    gr[0] = g_um2;
    gr[1] = g_um1;
    gr[2] = g_u0;
    gr[3] = g_up1;
    gr[4] = g_up2;
}

template <class T>
__device__ __noinline__ void scatter_weno(const DevProb<T>& P, const mol_term& tm, const T* u, T* lam, const int* I, T g,
                                          T t, const T* p) {
    const int f = tm.field, d = tm.dim, n = P.n[d];
    int J[3] = {I[0], I[1], I[2]};
    T v[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        J[d] = wrap_periodic(I[d] - 2 + k, n);
        v[k] = load_pt(P, u, f, J[0], J[1], J[2], t, p);
    }
    T gr[5];
    weno5_grad<T>(v[0], v[1], v[2], v[3], v[4], T(tm.eps), T(tm.dx), gr);
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        J[d] = wrap_periodic(I[d] - 2 + k, n);
        scatter_pt(P, lam, f, J[0], J[1], J[2], g * gr[k], t, p);
    }
}

}  // namespace mol
