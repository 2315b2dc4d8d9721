// Device side of the method-of-lines hot path: problem view, tap selection,
// boundary rows, derivative terms and the register-machine interpreter of the
// pointwise programs.  Templated on the state type T (double, or float for the
// Float32-state variant).
//
// GB300 note: sm_103a executes FP64 at 1/64 of its FP32 rate, so every kernel in
// this library is bound by the FP64 pipe long before HBM.  Integer work (tap
// selection, interpreter dispatch, index wrapping) issues on other pipes and is
// effectively free next to one warp-wide DFMA; the design therefore spends
// integer instructions to save FP64 ones (host-hoisted coordinate terms, shared
// reciprocals in WENO, Markstein division by 3).
#pragma once

#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#include <stdint.h>
#endif

#include "molgpu.h"

// Generated modules compile the rows their problem has: edge-aligned face rows and
// extrapolated points only when some boundary row uses them (each adds out-of-line code
// that the stage kernels' register allocation pays for).  The library's own kernels
// (the interpreter) always have both.
#ifndef MOL_JIT
#define MOL_HAS_EDGE_ROWS 1
#define MOL_HAS_EXTRAP_ROWS 1
#endif
#ifndef MOL_HAS_EDGE_ROWS
#define MOL_HAS_EDGE_ROWS 0
#endif
#ifndef MOL_HAS_EXTRAP_ROWS
#define MOL_HAS_EXTRAP_ROWS 0
#endif

namespace mol {

// Device-resident integrator state; kernels read t/dt from here so a captured
// CUDA graph can be replayed step after step.
struct SolverState {
    double t, dt, t1, abstol, reltol;
    double qold, EEst, dtmin;
    double dta[8][8];   // dt * a_ij of the Tsit5 tableau (row = stage index)
    double dtb[8];      // dt * btilde_j
    double sums[4];
    long long naccept, nreject, nf, iter, maxiters;
    int done, status, accepted;
    int nonfinite;      // set by the last SSPRK33 stage when a state value is NaN or Inf (sticky)
    unsigned int blocks_done, pad2;
};

// One boundary row.  For rows with constant coefficients (prog < 0) the host also
// stores inv = 1 / (a + b w_kb) (Robin/Neumann: the boundary value is
// (g - b sum_{k != kb} w_k u_k) * inv) and c0 = g / a (Dirichlet, b == 0).  xop >= 0: the
// point next to the boundary point is observed too, through row 1 of that operator's
// low (high) extrapolation table (generate_extrap_eqs!, generate_bc_eqs.jl:336-392).
template <class T>
struct DevBC {
    int kind, prog, op, xop;
    int iop, pad;  // MOL_BC_EDGE: interpolation operator (op: half-offset first derivative)
    T a, b, g;
    T inv, c0;
};

// Everything a kernel needs to evaluate f(du, u, p, t) of one problem instance.
// Passed by value (kernel parameter space / constant bank); arrays live in HBM.
template <class T>
struct DevProb {
    int ndim, nfields, nparams, cell_prog;
    int n[3];        // grid points per dim (1 for unused dims)
    int lo[3], up[3];
    int ni[3];       // interior extents
    int permask[MOL_MAX_FIELDS];  // bit d set: field periodic along d
    long long ncell; // interior cells per field
    const T* coords[3];
    const DevBC<T>* bc;           // [field][dim][side]
    const mol_op1d* ops;
    const T* w;
    const mol_term* terms;
    const mol_instr* code;
    const int* progs;             // (start, len) pairs
    const T* consts;
    const T* aux;
    const long long* aux_off;     // naux + 1 offsets into aux
    int naux;
    // left faces of the nonlinear-Laplacian terms from the face pass ([slot][cell]), or null;
    // slot q of cell c at faces[q * fstride + c] (fstride = ncell for the face pass over the
    // whole grid; the ensemble kernel points faces at a shared-memory window of fstride cells)
    const T* faces;
    long long fstride;
    long long fbeg, fend;   // cells whose faces `faces` holds: [fbeg, fend)
    // per-cell coefficient arrays of the generated cell's coefficient stencils ([array][cell],
    // filled by k_coef_t at plan creation), or null (ensembles; the interpreter)
    const T* cw;
    // cell index -> grid position by multiplication (divmagic) when ncell < 2^31: the magic
    // multipliers and shifts of ni[0] and ni[1]
    unsigned dm[2], ds[2];
    int fastdiv;
};

// Division of n < 2^31 by an invariant divisor d with a precomputed multiplier m and shift l
// (Granlund and Montgomery, "Division by invariant integers using multiplication", PLDI
// 1994, Fig. 4.1 with N = 32): l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, and
// floor(n / d) = (umulhi(m, n) + n) >> l, the sum below 2^32 for n < 2^31.  Grid positions
// are taken from cell indices in every kernel; the hardware has no integer divide, and the
// generic 64-bit division costs ~100 instructions per cell, as much as a face pass's FP64 work.
__host__ __device__ inline void divmagic(unsigned d, unsigned* m, unsigned* l) {
    unsigned s = 0;
    while (s < 32 && (1ull << s) < (unsigned long long)d) ++s;
    *l = s;
    *m = (unsigned)((((1ull << s) - d) << 32) / d + 1);
}
__device__ __forceinline__ unsigned divq(unsigned n, unsigned m, unsigned l) { return (__umulhi(m, n) + n) >> l; }

__device__ __forceinline__ int wrap_periodic(int i, int l) {
    // _wrapperiodic (interface_boundary.jl:33-42): u[1] == u[l]
    return i <= 1 ? i + (l - 1) : (i > l ? i - (l - 1) : i);
}

// True when `p` holds on every lane converged here.  The generated terms branch on it:
// FP64 instructions cost the same however few lanes are active, so a warp that straddles
// an edge runs the edge path for all its lanes (it also gives interior cells their exact
// result) instead of both paths one after the other.
__device__ __forceinline__ bool warp_all(bool p) { return __all_sync(__activemask(), p); }

// A product rounded on its own, never contracted into an FMA with the addition that uses it:
// the folded nonlinear-Laplacian faces are stored by the face pass (rounded) and subtracted
// in the cell, so the cells' own evaluation must round them the same way to agree bit for bit.
__device__ __forceinline__ double mulrn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mulrn(float a, float b) { return __fmul_rn(a, b); }

// Offset, along a periodic line of n points, of the tap at i + off after the same single
// wrap (the unknowns being points 2..n).  Valid while |off| <= n - 2.
__device__ __forceinline__ int wrap_off(int i, int off, int n) {
    const int q = i + off;
    return q <= 1 ? off + (n - 1) : (q > n ? off - (n - 1) : off);
}

// True when dimension d of field f is periodic with unknowns 2..n and at least `reach`
// points beyond every tap offset, so every cell can use interior weights with wrapped
// offsets (the same for the whole grid: a uniform branch).
template <class T>
__device__ __forceinline__ bool wrap_line_ok(const DevProb<T>& P, int f, int d, int reach) {
    return ((P.permask[f] >> d) & 1) && P.lo[d] == 1 && P.up[d] == 0 && P.n[d] - 2 >= reach;
}

template <class T>
__device__ __forceinline__ long long flat_interior(const DevProb<T>& P, int i0, int i1, int i2) {
    return (long long)(i0 - 1 - P.lo[0]) +
           (long long)P.ni[0] * ((long long)(i1 - 1 - P.lo[1]) + (long long)P.ni[1] * (long long)(i2 - 1 - P.lo[2]));
}

// Interior-or-zero load (no boundary row evaluation): used inside boundary rows.
template <class T>
__device__ __forceinline__ T load_interior(const DevProb<T>& P, const T* u, int f, const int* I) {
    bool in = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) in &= (I[d] > P.lo[d]) & (I[d] <= P.n[d] - P.up[d]);
    if (!in) return T(0);
    return u[(long long)f * P.ncell + flat_interior(P, I[0], I[1], I[2])];
}

struct TapSel {
    long long woff;
    int first, cnt;
    bool wrap;
};

// Tap selection of one 1-D operator at position i of a line of `len` points.
__device__ __forceinline__ TapSel select_taps(const mol_op1d& op, int i, int len, bool per) {
    TapSel s;
    if (!per && i <= op.nlo) {
        const int ti = i < 1 ? 0 : i - 1;  // positions below 1 only occur in malformed descriptors
        s.woff = op.w_lo + (long long)ti * op.bLlo; s.first = 1; s.cnt = op.bLlo; s.wrap = false;
    } else if (!per && i > len - op.nhi) {
        int ti = len - i - op.hi_base;
        ti = ti < 0 ? 0 : ti;
        s.woff = op.w_hi + (long long)ti * op.bLhi; s.first = len - op.bLhi + 1;
        s.cnt = op.bLhi; s.wrap = false;
    } else {
        s.woff = op.w_int; s.first = i + op.omin; s.cnt = op.L; s.wrap = per;
        if (op.nrows > 0) {  // per-point rows (nonuniform grid): the row of point i, kept in range
            int r = i - op.nlo - 1;
            r = r < 0 ? 0 : (r >= op.nrows ? op.nrows - 1 : r);
            s.woff += (long long)r * op.L;
        }
    }
    return s;
}

// Elementary functions, comparisons and integer powers of the programs.
template <class T>
__device__ __forceinline__ T apply_fn(int fn, T x) {
    switch (fn) {
        case MOL_FN_SIN: return sin(x);
        case MOL_FN_COS: return cos(x);
        case MOL_FN_TAN: return tan(x);
        case MOL_FN_EXP: return exp(x);
        case MOL_FN_LOG: return log(x);
        case MOL_FN_SQRT: return sqrt(x);
        case MOL_FN_ABS: return fabs(x);
        case MOL_FN_TANH: return tanh(x);
        case MOL_FN_SINH: return sinh(x);
        case MOL_FN_COSH: return cosh(x);
        case MOL_FN_ATAN: return atan(x);
        default: return x;
    }
}

template <class T>
__device__ __forceinline__ T apply_cmp(int c, T a, T b) {
    bool r;
    switch (c) {
        case MOL_CMP_LE: r = a <= b; break;
        case MOL_CMP_LT: r = a < b; break;
        case MOL_CMP_GE: r = a >= b; break;
        case MOL_CMP_GT: r = a > b; break;
        default: r = a == b; break;
    }
    return r ? T(1) : T(0);
}

template <class T>
__device__ __forceinline__ T powi(T x, int n) {
    if (n == 2) return x * x;
    if (n == 3) return x * x * x;
    if (n == 1) return x;
    if (n == 0) return T(1);
    if (n == -1) return T(1) / x;
    if (n == -2) return T(1) / (x * x);
    return pow(x, T(n));
}

// Small straight-line program used by boundary rows (a, b, g may depend on t, x, p).
template <class T>
__device__ T run_bc_prog(const DevProb<T>& P, int prog, int out_index, const int* I, T t, const T* p) {
    T r[16];
    const int start = P.progs[2 * prog], len = P.progs[2 * prog + 1];
    T res = T(0);
    for (int pc = start; pc < start + len; ++pc) {
        const mol_instr in = P.code[pc];
        const int dst = in.dst & 15;
        switch (in.op) {
            case MOL_OP_CONST: r[dst] = P.consts[in.imm]; break;
            case MOL_OP_PARAM: r[dst] = p[in.imm]; break;
            case MOL_OP_COORD: r[dst] = P.coords[in.imm][I[in.imm] - 1]; break;
            case MOL_OP_TIME: r[dst] = t; break;
            case MOL_OP_AUX:  // a full-grid array (host-evaluated registered function) at the point
                r[dst] = P.aux[P.aux_off[in.imm] + (long long)(I[0] - 1) +
                               (long long)P.n[0] * ((long long)(I[1] - 1) + (long long)P.n[1] * (I[2] - 1))];
                break;
            case MOL_OP_ADD: r[dst] = r[in.a & 15] + r[in.b & 15]; break;
            case MOL_OP_SUB: r[dst] = r[in.a & 15] - r[in.b & 15]; break;
            case MOL_OP_MUL: r[dst] = r[in.a & 15] * r[in.b & 15]; break;
            case MOL_OP_DIV: r[dst] = r[in.a & 15] / r[in.b & 15]; break;
            case MOL_OP_NEG: r[dst] = -r[in.a & 15]; break;
#if !defined(MOL_JIT) || defined(MOL_BC_FULL_OPS)
            // Elementary functions in a boundary program: compiled into generated code only when
            // some boundary program uses them (their range reduction would otherwise raise the
            // register count of every stage kernel that can reach a boundary row).
            case MOL_OP_POWI: r[dst] = powi(r[in.a & 15], in.imm); break;
            case MOL_OP_POW: r[dst] = pow(r[in.a & 15], r[in.b & 15]); break;
            case MOL_OP_FN: r[dst] = apply_fn(in.imm, r[in.a & 15]); break;
            case MOL_OP_CMP: r[dst] = apply_cmp(in.imm, r[in.a & 15], r[in.b & 15]); break;
            case MOL_OP_IFELSE: r[dst] = r[in.a & 15] != T(0) ? r[in.b & 15] : r[in.c & 15]; break;
#endif
            case MOL_OP_OUT: if (in.imm == out_index) res = r[in.a & 15]; break;
            default: break;
        }
    }
    return res;
}

// Value of field f at full-grid point I (1-based), resolving boundary rows:
// unknowns are read directly, a point outside the interior in exactly one
// dimension is an observed boundary value (Robin/Neumann/Dirichlet row,
// generate_bc_eqs.jl:238-328, solved for the boundary point), a point outside
// in two or more dimensions is a corner row (~ 0, generate_bc_eqs.jl:396-459).
template <class T>
__device__ __noinline__ T bc_value(const DevProb<T>& P, const T* u, int f, int* I, int dout, int side, T t, const T* p);

template <class T>
__device__ __forceinline__ T load_pt(const DevProb<T>& P, const T* u, int f, int i0, int i1, int i2, T t, const T* p) {
    int I[3] = {i0, i1, i2};
    int nout = 0, dout = 0, side = 0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        if ((P.permask[f] >> d) & 1) I[d] = wrap_periodic(I[d], P.n[d]);
        // anything still outside the interior (including a tap that one wrap did not bring
        // back) resolves through the boundary rows below and is never dereferenced
        if (I[d] <= P.lo[d]) {
            ++nout; dout = d; side = 0;
        } else if (I[d] > P.n[d] - P.up[d]) {
            ++nout; dout = d; side = 1;
        }
    }
    if (nout == 0) return u[(long long)f * P.ncell + flat_interior(P, I[0], I[1], I[2])];
    if (nout > 1) return T(0);
    return bc_value(P, u, f, I, dout, side, t, p);
}

template <class T>
__device__ __noinline__ T bc_row_value(const DevProb<T>& P, const T* u, int f, int* I, int dout, int side, T t,
                                       const T* p);

// Extrapolation row of the point next to the boundary point (point 2, or n-1): the
// second low (high) row of BoundaryInterpolatorExtrapolator(q) over the first (last) q
// points, its own slot zero, the boundary point through its (Dirichlet) row
// (generate_extrap_eqs!, generate_bc_eqs.jl:336-392; extrapolation_weights.jl:1-60).
template <class T>
__device__ __forceinline__ T extrap_value(const DevProb<T>& P, const T* u, int f, int* I, int dout, int side, T t,
                                          const T* p) {
    const DevBC<T>& B = P.bc[(f * 3 + dout) * 2 + side];
    const mol_op1d& x = P.ops[B.xop];
    const int n = P.n[dout], self = I[dout];
    const T* w = side == 0 ? P.w + x.w_lo + x.bLlo : P.w + x.w_hi + x.bLhi;
    const int first = side == 0 ? 1 : n - x.bLhi + 1;
    const int cnt = side == 0 ? x.bLlo : x.bLhi;
    const int qb = side == 0 ? 1 : n;
    int J[3] = {I[0], I[1], I[2]};
    T acc = T(0);
    bool started = false;
    for (int k = 0; k < cnt; ++k) {
        const int q = first + k;
        if (q == self) continue;
        J[dout] = q;
        const T v = q == qb ? bc_row_value(P, u, f, J, dout, side, t, p) : load_interior(P, u, f, J);
        acc = started ? fma(w[k], v, acc) : w[k] * v;
        started = true;
    }
    return acc;
}

template <class T>
__device__ __noinline__ T bc_value(const DevProb<T>& P, const T* u, int f, int* I, int dout, int side, T t, const T* p) {
    const int i = I[dout], n = P.n[dout];
    if ((side == 0 && i == 1) || (side == 1 && i == n)) return bc_row_value(P, u, f, I, dout, side, t, p);
#if MOL_HAS_EXTRAP_ROWS
    if (P.bc[(f * 3 + dout) * 2 + side].xop >= 0 && ((side == 0 && i == 2) || (side == 1 && i == n - 1)))
        return extrap_value(P, u, f, I, dout, side, t, p);
#endif
    return T(0);
}

// Edge-aligned grid: a * sum_k c_k u_k + b * sum_k d_k u_k = g at the face between the ghost
// point and the first (last) unknown, c the interpolation and d the half-offset derivative
// table at position 1 (n-1), solved for the ghost point (boundary_value_maps for
// EdgeAlignedGrid, generate_bc_eqs.jl:80-160; tables selected as in
// half_offset_centred_difference.jl:9-37).
// Scalar coordinates (no pointer to a caller's array): the generated stage kernels reach it
// from their line helpers, and an address-taken array there costs them a stack frame.
template <class T>
__device__ __noinline__ T edge_row_value(const DevProb<T>& P, const T* u, int f, int i0, int i1, int i2, int dout,
                                         int side, T t, const T* p) {
    const int I[3] = {i0, i1, i2};
    const DevBC<T>& B = P.bc[(f * 3 + dout) * 2 + side];
    T a = B.a, b = B.b, g = B.g;
    if (B.prog >= 0) {
        a = run_bc_prog(P, B.prog, 0, I, t, p);
        b = run_bc_prog(P, B.prog, 1, I, t, p);
        g = run_bc_prog(P, B.prog, 2, I, t, p);
    }
    const int n = P.n[dout], pos = side == 0 ? 1 : n - 1, ghost = side == 0 ? 1 : n;
    const TapSel si = select_taps(P.ops[B.iop], pos, n, false);
    const TapSel sd = select_taps(P.ops[B.op], pos, n, false);
    int J[3] = {I[0], I[1], I[2]};
    T sum_i = T(0), sum_d = T(0), wi = T(0), wd = T(0);
    for (int k = 0; k < si.cnt; ++k) {
        const int q = si.first + k;
        if (q == ghost) { wi = P.w[si.woff + k]; continue; }
        J[dout] = q;
        sum_i = fma(P.w[si.woff + k], load_interior(P, u, f, J), sum_i);
    }
    for (int k = 0; k < sd.cnt; ++k) {
        const int q = sd.first + k;
        if (q == ghost) { wd = P.w[sd.woff + k]; continue; }
        J[dout] = q;
        sum_d = fma(P.w[sd.woff + k], load_interior(P, u, f, J), sum_d);
    }
    return (g - a * sum_i - b * sum_d) / (a * wi + b * wd);
}

template <class T>
__device__ __noinline__ T bc_row_value(const DevProb<T>& P, const T* u, int f, int* I, int dout, int side, T t,
                                       const T* p) {
    const DevBC<T> B = P.bc[(f * 3 + dout) * 2 + side];
#if MOL_HAS_EDGE_ROWS
    if (B.kind == MOL_BC_EDGE) return edge_row_value(P, u, f, I[0], I[1], I[2], dout, side, t, p);
#endif
    if (B.kind != MOL_BC_ROBIN) return T(0);
    const bool dyn = B.prog >= 0;
    T a = B.a, b = B.b, g = B.g;
    if (dyn) {
        a = run_bc_prog(P, B.prog, 0, I, t, p);
        b = run_bc_prog(P, B.prog, 1, I, t, p);
        g = run_bc_prog(P, B.prog, 2, I, t, p);
    }
    if (b == T(0)) return dyn ? g / a : B.c0;
    const mol_op1d op = P.ops[B.op];
    const int n = P.n[dout];
    const T* w = side == 0 ? P.w + op.w_lo : P.w + op.w_hi;  // centered table at the last point
    const int first = side == 0 ? 1 : n - op.bLhi + 1;
    const int cnt = side == 0 ? op.bLlo : op.bLhi;
    const int kb = side == 0 ? 0 : cnt - 1;
    T acc = T(0);
    bool started = false;
    int J[3] = {I[0], I[1], I[2]};
    for (int k = 0; k < cnt; ++k) {
        if (k == kb) continue;
        J[dout] = first + k;
        const T term = w[k] * load_interior(P, u, f, J);
        acc = started ? acc + term : term;
        started = true;
    }
    return dyn ? (g - b * acc) / (a + b * w[kb]) : (g - b * acc) * B.inv;
}

// sum_k w_k u[tap_k] along dimension d at position `pos` of a line of `len` points
// (centered_difference.jl:5-30, upwind_difference.jl:1-28, half_offset_centred_difference.jl:9-37).
template <class T>
__device__ T apply_op_at(const DevProb<T>& P, const mol_op1d& op, const T* u, int f, int d, const int* I, int pos,
                         int len, T t, const T* p) {
    const bool per = (P.permask[f] >> d) & 1;
    const TapSel s = select_taps(op, pos, len, per);
    int J[3] = {I[0], I[1], I[2]};
    T acc = T(0);
    for (int k = 0; k < s.cnt; ++k) {
        int tp = s.first + k;
        if (per) tp = wrap_periodic(tp, P.n[d]);
        J[d] = tp;
        const T v = load_pt(P, u, f, J[0], J[1], J[2], t, p);
        acc = k == 0 ? P.w[s.woff] * v : fma(P.w[s.woff + k], v, acc);
    }
    return acc;
}

template <class T>
__device__ __forceinline__ T apply_op(const DevProb<T>& P, const mol_op1d& op, const T* u, int f, int d, const int* I,
                                      T t, const T* p) {
    return apply_op_at(P, op, u, f, d, I, I[d], P.n[d], t, p);
}

// Stride of dimension d in the interior (unknown) layout.
template <class T>
__device__ __forceinline__ long long gstride(const DevProb<T>& P, int d) {
    return d == 0 ? 1ll : (d == 1 ? (long long)P.ni[0] : (long long)P.ni[0] * P.ni[1]);
}

// ---------------------------------------------------------------------------
// Line helpers for 1-D terms along a compile-time dimension D.  The cell being
// evaluated is an unknown, so only the coordinate along D can leave the interior,
// and an interior tap sits at a fixed flat offset from the cell's own index c.
// Loops over taps are unrolled to the operator's largest tap count NT (known when
// the code is generated), so a cell near an edge issues its loads together
// instead of walking them one call at a time.

// Boundary value of field f at the end `side` of the line through the cell: the
// observed boundary row solved for the boundary point (same arithmetic as bc_value).
// Out of line (edge cells only; inlined into every tap it multiplies compile time
// several-fold) and with scalar arguments, so callers keep their index arrays in
// registers.  DYN: some boundary row of this field along D has coefficients given by
// a program (time or coordinate dependent); only then is bc_value reachable.
template <class T, int D, bool DYN>
__device__ __noinline__ T bc_line_value(const DevProb<T>& P, const T* __restrict__ u, int f, int i0, int i1, int i2,
                                        long long c, int side, T t, const T* __restrict__ p) {
    const int iD = D == 0 ? i0 : (D == 1 ? i1 : i2);
    const DevBC<T>& B = P.bc[(f * 3 + D) * 2 + side];
#if MOL_HAS_EDGE_ROWS
    if (B.kind == MOL_BC_EDGE) {
        const int e = side == 0 ? 1 : P.n[D];
        return edge_row_value(P, u, f, D == 0 ? e : i0, D == 1 ? e : i1, D == 2 ? e : i2, D, side, t, p);
    }
#endif
    if (B.kind != MOL_BC_ROBIN) return T(0);
    if (DYN && B.prog >= 0) {
        int J[3] = {i0, i1, i2};
        J[D] = side == 0 ? 1 : P.n[D];
        return bc_value(P, u, f, J, D, side, t, p);
    }
    if (B.b == T(0)) return B.c0;
    const mol_op1d& op = P.ops[B.op];
    const int n = P.n[D];
    const T* __restrict__ w = side == 0 ? P.w + op.w_lo : P.w + op.w_hi;
    const int first = side == 0 ? 1 : n - op.bLhi + 1;
    const int cnt = side == 0 ? op.bLlo : op.bLhi;
    const int kb = side == 0 ? 0 : cnt - 1;
    const long long s = gstride(P, D);
    const T* __restrict__ uf = u + (long long)f * P.ncell + c;
    T acc = T(0);
    bool started = false;
#pragma unroll 4
    for (int k = 0; k < cnt; ++k) {
        if (k == kb) continue;
        const int q = first + k;
        const T v = (q > P.lo[D] && q <= n - P.up[D]) ? uf[(long long)(q - iD) * s] : T(0);
        const T term = w[k] * v;
        acc = started ? acc + term : term;
        started = true;
    }
    return (B.g - B.b * acc) * B.inv;
}

// Extrapolated point next to the boundary point of the line through the cell (extrap_value
// restricted to D).
template <class T, int D, bool DYN>
__device__ __noinline__ T extrap_line_value(const DevProb<T>& P, const T* __restrict__ u, int f, int i0, int i1,
                                            int i2, long long c, int side, T t, const T* __restrict__ p) {
    const int iD = D == 0 ? i0 : (D == 1 ? i1 : i2);
    const DevBC<T>& B = P.bc[(f * 3 + D) * 2 + side];
    if (B.xop < 0) return T(0);
    const mol_op1d& x = P.ops[B.xop];
    const int n = P.n[D];
    const T* __restrict__ w = side == 0 ? P.w + x.w_lo + x.bLlo : P.w + x.w_hi + x.bLhi;
    const int first = side == 0 ? 1 : n - x.bLhi + 1;
    const int cnt = side == 0 ? x.bLlo : x.bLhi;
    const int self = side == 0 ? 2 : n - 1, qb = side == 0 ? 1 : n;
    const long long s = gstride(P, D);
    const T* __restrict__ uf = u + (long long)f * P.ncell + c;
    T acc = T(0);
    bool started = false;
    for (int k = 0; k < cnt; ++k) {
        const int q = first + k;
        if (q == self) continue;
        T v;
        if (q == qb) v = bc_line_value<T, D, DYN>(P, u, f, i0, i1, i2, c, side, t, p);
        else v = (q > P.lo[D] && q <= n - P.up[D]) ? uf[(long long)(q - iD) * s] : T(0);
        acc = started ? fma(w[k], v, acc) : w[k] * v;
        started = true;
    }
    return acc;
}

// A point of the line through the cell that is not an unknown: a boundary point, the
// extrapolated point next to it, or nothing (0).  One out-of-line call per tap, so the
// generated kernels that inline line_pt keep a single call site per tap.
template <class T, int D, bool DYN>
__device__ __noinline__ T line_edge_pt(const DevProb<T>& P, const T* __restrict__ u, int f, int i0, int i1, int i2,
                                       long long c, int q, T t, const T* __restrict__ p) {
    const int n = P.n[D];
    if (q <= P.lo[D]) {
        if (q == 1) return bc_line_value<T, D, DYN>(P, u, f, i0, i1, i2, c, 0, t, p);
#if MOL_HAS_EXTRAP_ROWS
        if (q == 2) return extrap_line_value<T, D, DYN>(P, u, f, i0, i1, i2, c, 0, t, p);
#endif
        return T(0);
    }
    if (q == n) return bc_line_value<T, D, DYN>(P, u, f, i0, i1, i2, c, 1, t, p);
#if MOL_HAS_EXTRAP_ROWS
    if (q == n - 1) return extrap_line_value<T, D, DYN>(P, u, f, i0, i1, i2, c, 1, t, p);
#endif
    return T(0);
}

// Field f at full-grid position q of the line through the cell (load_pt restricted to D).
template <class T, int D, bool DYN>
__device__ __forceinline__ T line_pt(const DevProb<T>& P, const T* __restrict__ u, int f, const int* I, long long c,
                                     int q, T t, const T* __restrict__ p) {
    const int n = P.n[D];
    if ((P.permask[f] >> D) & 1) q = wrap_periodic(q, n);
    if (q > P.lo[D] && q <= n - P.up[D])
        return u[(long long)f * P.ncell + c + (long long)(q - I[D]) * gstride(P, D)];
    return line_edge_pt<T, D, DYN>(P, u, f, I[0], I[1], I[2], c, q, t, p);
}

// apply_op_at restricted to D: sum_k w_k u[tap_k] at position `pos` of a line of `len` points.
template <class T, int D, int NT, bool DYN>
__device__ __forceinline__ T apply_op_line(const DevProb<T>& P, const mol_op1d& op, const T* __restrict__ u, int f,
                                           const int* I, long long c, int pos, int len, T t,
                                           const T* __restrict__ p) {
    const bool per = (P.permask[f] >> D) & 1;
    const TapSel s = select_taps(op, pos, len, per);
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        if (k < s.cnt) {
            const T v = line_pt<T, D, DYN>(P, u, f, I, c, s.first + k, t, p);
            acc = k == 0 ? P.w[s.woff] * v : fma(P.w[s.woff + k], v, acc);
        }
    }
    return acc;
}

// The five WENO taps of the cell along D (weno_taps restricted to D).
template <class T, int D, bool DYN>
__device__ __forceinline__ void weno_taps_line(const DevProb<T>& P, int f, const T* __restrict__ u, const int* I,
                                               long long c, T t, const T* __restrict__ p, T v[5]) {
#pragma unroll
    for (int k = 0; k < 5; ++k) v[k] = line_pt<T, D, DYN>(P, u, f, I, c, I[D] - 2 + k, t, p);
}

// True when operator `o` at position i of dimension d uses its interior weights and
// every tap is an unknown of the same line without wrapping: the generated code
// then reads the taps at compile-time offsets.
template <class T>
__device__ __forceinline__ bool fast_line(const DevProb<T>& P, const mol_op1d& o, int f, int d, int i) {
    const int first = i + o.omin, last = first + o.L - 1;
    if ((P.permask[f] >> d) & 1) return first > P.lo[d] && last <= P.n[d];
    return i > o.nlo && i <= P.n[d] - o.nhi && first > P.lo[d] && last <= P.n[d] - P.up[d];
}

template <class T>
__device__ __forceinline__ bool fast_weno(const DevProb<T>& P, int f, int d, int i) {
    return i - 2 > P.lo[d] && i + 2 <= P.n[d] - P.up[d];
}

// Nonlinear Laplacian at i: the outer half-offset stencil (position i-1 on n-1 points) uses
// interior weights and every face's inner derivative and interpolation do too.
template <class T>
__device__ __forceinline__ bool fast_nonlinlap(const DevProb<T>& P, const mol_op1d& oo, const mol_op1d& oi,
                                               const mol_op1d& op, int f, int d, int i) {
    const bool per = (P.permask[f] >> d) & 1;
    const int pos = i - 1;
    if (!per && !(pos > oo.nlo && pos <= (P.n[d] - 1) - oo.nhi)) return false;
    for (int m = 0; m < oo.L; ++m) {
        const int Ih = pos + oo.omin + m;
        if (!fast_line(P, oi, f, d, Ih) || !fast_line(P, op, f, d, Ih)) return false;
    }
    return true;
}

// Face arrays have npts[d] + 1 entries along d (half point Ih + 1/2 at index Ih) and the
// full grid extents elsewhere.
template <class T>
__device__ __forceinline__ long long face_index(const DevProb<T>& P, int d, int Ih, const int* I) {
    Ih = Ih < 0 ? 0 : (Ih > P.n[d] ? P.n[d] : Ih);
    const long long e0 = P.n[0] + (d == 0), e1 = P.n[1] + (d == 1);
    const long long j0 = d == 0 ? Ih : I[0] - 1, j1 = d == 1 ? Ih : I[1] - 1, j2 = d == 2 ? Ih : I[2] - 1;
    return j0 + e0 * (j1 + e1 * j2);
}

// Mixed derivative: tensor product of two first-derivative centered stencils
// (2nd_order_mixed_deriv.jl:5-22), both wrapped.
template <class T>
__device__ T apply_mixed(const DevProb<T>& P, const mol_term& tm, const T* u, const int* I, T t, const T* p) {
    const int f = tm.field, d1 = tm.dim, d2 = tm.dim2;
    const mol_op1d o1 = P.ops[tm.op], o2 = P.ops[tm.op2];
    const bool p1 = (P.permask[f] >> d1) & 1, p2 = (P.permask[f] >> d2) & 1;
    const TapSel s1 = select_taps(o1, I[d1], P.n[d1], p1);
    const TapSel s2 = select_taps(o2, I[d2], P.n[d2], p2);
    int J[3] = {I[0], I[1], I[2]};
    T acc = T(0);
    bool started = false;
    for (int a = 0; a < s1.cnt; ++a) {
        const T wa = P.w[s1.woff + a];
        if (wa == T(0)) continue;  // zero taps drop out of the symbolic sum
        int ta = s1.first + a;
        if (s1.wrap) ta = wrap_periodic(ta, P.n[d1]);
        J[d1] = ta;
        for (int b = 0; b < s2.cnt; ++b) {
            const T wb = P.w[s2.woff + b];
            if (wb == T(0)) continue;
            int tb = s2.first + b;
            if (s2.wrap) tb = wrap_periodic(tb, P.n[d2]);
            J[d2] = tb;
            const T v = load_pt(P, u, f, J[0], J[1], J[2], t, p);
            const T ww = wa * wb;
            acc = started ? fma(ww, v, acc) : ww * v;
            started = true;
        }
    }
    return acc;
}

// Jiang-Shu WENO5 node derivative (WENO.jl:6-57), periodic taps i-2..i+2.
// Algebraically identical to the reference.  In FP64 the six nonlinear weights
// gamma_k / (eps + beta_k)^2 are brought to the common denominator
// prod_j (eps + beta_j)^2, so (hp - hm) costs one division instead of the twelve
// the reference spells out; eps >= 1e-6 keeps every product far from underflow.
// FP32 keeps the reciprocal form (the products would underflow in float).
template <class T>
__device__ __forceinline__ T weno5_point(T um2, T um1, T u0, T up1, T up2, T eps, T inv_dx) {
    const T c13_12 = T(13) / T(12);
    if (sizeof(T) == 8) {
        // FP64 issue is the bound: beta_1 and beta_3 take their second square as (b/2)^2 with b/2
        // formed directly (1.5 u - 2 u' + 0.5 u''), bit for bit 0.25 b^2 since scaling by 1/2
        // commutes with rounding; the ideal weights (0.1, 0.6, 0.3) ride on the candidate
        // reconstructions' coefficients instead of six products with the P_k.  u - 2 u' is
        // fma(-2, u', u) (2 u' is exact: the same rounded difference), and eps enters through
        // the FMA of the second square instead of a separate addition (eps + beta_k rounded in
        // another order: one instruction fewer per indicator)
        const T a1 = fma(T(-2), up1, u0) + up2, h1 = T(1.5) * u0 - T(2) * up1 + T(0.5) * up2;
        const T a2 = fma(T(-2), u0, um1) + up1, b2 = um1 - up1;
        const T a3 = fma(T(-2), um1, um2) + u0, h3 = T(0.5) * um2 - T(2) * um1 + T(1.5) * u0;
        const T e1 = fma(c13_12 * a1, a1, fma(h1, h1, eps));
        const T e2 = fma(c13_12 * a2, a2, fma(T(0.25) * b2, b2, eps));
        const T e3 = fma(c13_12 * a3, a3, fma(h3, h3, eps));
        const T s1 = e1 * e1, s2 = e2 * e2, s3 = e3 * e3;
        const T P1 = s2 * s3, P2 = s1 * s3, P3 = s1 * s2;   // P_k = prod_{j != k} (eps + beta_j)^2
        // gamma_k times the candidates (scaled by 6, the 1/6 folded into inv_dx below)
        const T gm1 = T(1.1) * u0 - T(0.7) * up1 + T(0.2) * up2;   // 0.1 (11 u0 - 7 up1 + 2 up2)
        const T gm2 = T(3.0) * u0 - T(0.6) * up1 + T(1.2) * um1;   // 0.6 (5 u0 - up1 + 2 um1)
        const T gm3 = T(0.6) * u0 + T(1.5) * um1 - T(0.3) * um2;   // 0.3 (2 u0 + 5 um1 - um2)
        const T gp1 = T(0.6) * u0 + T(1.5) * up1 - T(0.3) * up2;   // 0.3 (2 u0 + 5 up1 - up2)
        const T gp2 = T(3.0) * u0 + T(1.2) * up1 - T(0.6) * um1;   // 0.6 (5 u0 + 2 up1 - um1)
        const T gp3 = T(1.1) * u0 - T(0.7) * um1 + T(0.2) * um2;   // 0.1 (11 u0 - 7 um1 + 2 um2)
        const T Np = fma(P1, gp1, fma(P2, gp2, P3 * gp3)), Dp = fma(T(0.3), P1, fma(T(0.6), P2, T(0.1) * P3));
        const T Nm = fma(P1, gm1, fma(P2, gm2, P3 * gm3)), Dm = fma(T(0.1), P1, fma(T(0.6), P2, T(0.3) * P3));
        return fma(Np, Dm, -Nm * Dp) / (Dp * Dm) * (inv_dx * T(1.0 / 6.0));
    }
    const T a1 = fma(T(-2), up1, u0) + up2, b1 = T(3) * u0 - T(4) * up1 + up2;
    const T a2 = fma(T(-2), u0, um1) + up1, b2 = um1 - up1;
    const T a3 = fma(T(-2), um1, um2) + u0, b3 = um2 - T(4) * um1 + T(3) * u0;
    const T e1 = eps + fma(c13_12 * a1, a1, T(0.25) * (b1 * b1));
    const T e2 = eps + fma(c13_12 * a2, a2, T(0.25) * (b2 * b2));
    const T e3 = eps + fma(c13_12 * a3, a3, T(0.25) * (b3 * b3));
    // candidate reconstructions, scaled by 6 (the common 1/6 is folded into inv_dx below)
    const T hm1 = T(11) * u0 - T(7) * up1 + T(2) * up2;
    const T hm2 = T(5) * u0 - up1 + T(2) * um1;
    const T hm3 = T(2) * u0 + T(5) * um1 - um2;
    const T hp1 = T(2) * u0 + T(5) * up1 - up2;
    const T hp2 = T(5) * u0 + T(2) * up1 - um1;
    const T hp3 = T(11) * u0 - T(7) * um1 + T(2) * um2;
    const T q1 = T(1) / (e1 * e1), q2 = T(1) / (e2 * e2), q3 = T(1) / (e3 * e3);
    const T wm1 = T(0.1) * q1, wm2 = T(0.6) * q2, wm3 = T(0.3) * q3;
    const T wp1 = T(0.3) * q1, wp2 = T(0.6) * q2, wp3 = T(0.1) * q3;
    const T hp = fma(wp1, hp1, fma(wp2, hp2, wp3 * hp3)) / (wp1 + wp2 + wp3);
    const T hm = fma(wm1, hm1, fma(wm2, hm2, wm3 * hm3)) / (wm1 + wm2 + wm3);
    return (hp - hm) * (inv_dx * T(1.0 / 6.0));
}

// The five WENO taps of a cell through the generic path (periodic wrap, observed
// boundary rows).  Kept inline so the generated code can load its taps on either
// path and then run the FP64 arithmetic once, with the warp converged.
template <class T>
__device__ __forceinline__ void weno_taps(const DevProb<T>& P, const mol_term& tm, const T* u, const int* I, T t,
                                          const T* p, T v[5]) {
    const int f = tm.field, d = tm.dim;
    int J[3] = {I[0], I[1], I[2]};
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        J[d] = I[d] - 2 + k;  // load_pt wraps along periodic dimensions
        v[k] = load_pt(P, u, f, J[0], J[1], J[2], t, p);
    }
}

// ---------------------------------------------------------------------------
// Node-centred Lagrange WENO-5 on a nonuniform dimension (nonuniform_weno.jl:120-163).
// `g` is the point's geometry row (56 values, see mol_term.variant); v the five taps.
// Per substencil k on taps k..k+2: r_k the derivative at the target, beta_k the Simpson
// smoothness indicator max(dx (dx/6)(pL^2 + 4 pM^2 + pR^2) + dx^3 dx pp^2, 0); the split
// ideal weights give the result sigma_p R_p - sigma_m R_m.

template <class T>
__device__ __forceinline__ T dot3(const T* w, const T* a) { return w[0] * a[0] + w[1] * a[1] + w[2] * a[2]; }

template <class T>
__device__ __forceinline__ T weno5nu_point(const T* __restrict__ g, const T v[5], T eps) {
    T b[3], r[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const T* m = g + 3 + 15 * k;
        const T* a = v + k;
        r[k] = dot3(m, a);
        const T pL = dot3(m + 3, a), pM = dot3(m + 6, a), pR = dot3(m + 9, a), pp = dot3(m + 12, a);
        const T I1 = g[0] * (pL * pL + T(4) * (pM * pM) + pR * pR);
        const T I2 = g[1] * (pp * pp);
        const T val = g[1] * I1 + g[2] * I2;
        b[k] = val > T(0) ? val : T(0);
    }
    T ap[3], am[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const T e = eps + b[k];
        const T e2 = e * e;
        ap[k] = g[48 + k] / e2;
        am[k] = g[51 + k] / e2;
    }
    const T sp = ap[0] + ap[1] + ap[2], sm = am[0] + am[1] + am[2];
    const T Rp = (ap[0] / sp) * r[0] + (ap[1] / sp) * r[1] + (ap[2] / sp) * r[2];
    const T Rm = (am[0] / sm) * r[0] + (am[1] / sm) * r[1] + (am[2] / sm) * r[2];
    return g[54] * Rp - g[55] * Rm;
}

// Value and gradient with respect to the five taps (reverse mode through the nonlinear
// weights: dF/dr_k = sp w+_k - sm w-_k, dF/dbeta_k = -2/(eps + beta_k) (sp w+_k (r_k - R+) -
// sm w-_k (r_k - R-)), beta_k quadratic in its three taps, zero where clipped).
template <class T>
__device__ __forceinline__ T weno5nu_valgrad(const T* __restrict__ g, const T v[5], T eps, T gr[5]) {
    T b[3], r[3], pl[3], pm[3], pr[3], pq[3];
    bool clip[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const T* m = g + 3 + 15 * k;
        const T* a = v + k;
        r[k] = dot3(m, a);
        pl[k] = dot3(m + 3, a);
        pm[k] = dot3(m + 6, a);
        pr[k] = dot3(m + 9, a);
        pq[k] = dot3(m + 12, a);
        const T I1 = g[0] * (pl[k] * pl[k] + T(4) * (pm[k] * pm[k]) + pr[k] * pr[k]);
        const T I2 = g[1] * (pq[k] * pq[k]);
        const T val = g[1] * I1 + g[2] * I2;
        clip[k] = !(val > T(0));
        b[k] = clip[k] ? T(0) : val;
    }
    T ap[3], am[3], ie[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const T e = eps + b[k];
        ie[k] = T(1) / e;
        const T e2 = e * e;
        ap[k] = g[48 + k] / e2;
        am[k] = g[51 + k] / e2;
    }
    const T sp = ap[0] + ap[1] + ap[2], sm = am[0] + am[1] + am[2];
    T wp[3], wm[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        wp[k] = ap[k] / sp;
        wm[k] = am[k] / sm;
    }
    const T Rp = wp[0] * r[0] + wp[1] * r[1] + wp[2] * r[2];
    const T Rm = wm[0] * r[0] + wm[1] * r[1] + wm[2] * r[2];
    const T SP = g[54], SM = g[55];
#pragma unroll
    for (int q = 0; q < 5; ++q) gr[q] = T(0);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const T* m = g + 3 + 15 * k;
        const T dr = SP * wp[k] - SM * wm[k];
        const T db = clip[k] ? T(0)
                             : T(-2) * ie[k] * (SP * wp[k] * (r[k] - Rp) - SM * wm[k] * (r[k] - Rm));
        // d beta / d a = dx (dx/6) (2 pL m1L + 8 pM m1M + 2 pR m1R) + dx^3 dx 2 pp m2M
        const T cL = db * g[1] * g[0] * T(2) * pl[k], cM = db * g[1] * g[0] * T(8) * pm[k];
        const T cR = db * g[1] * g[0] * T(2) * pr[k], cQ = db * g[2] * g[1] * T(2) * pq[k];
#pragma unroll
        for (int j = 0; j < 3; ++j)
            gr[k + j] += dr * m[j] + cL * m[3 + j] + cM * m[6 + j] + cR * m[9 + j] + cQ * m[12 + j];
    }
    return SP * Rp - SM * Rm;
}

// First tap of the nonuniform WENO stencil at point i of n (the two one-sided targets at
// each end, get_f_taps_coords with the scheme's boundary functions, WENO.jl:84-85).
__device__ __forceinline__ int weno_nu_first(int i, int n) { return i <= 2 ? 1 : (i > n - 2 ? n - 4 : i - 2); }

template <class T>
__device__ T apply_weno(const DevProb<T>& P, const mol_term& tm, const T* u, const int* I, T t, const T* p) {
    T v[5];
    if (tm.variant == 1) {
        const int d = tm.dim, n = P.n[d], q0 = weno_nu_first(I[d], n);
        int J[3] = {I[0], I[1], I[2]};
        for (int k = 0; k < 5; ++k) {
            J[d] = q0 + k;
            v[k] = load_pt(P, u, tm.field, J[0], J[1], J[2], t, p);
        }
        const mol_op1d& o = P.ops[tm.op];
        return weno5nu_point<T>(P.w + o.w_int + (long long)(I[d] - 1) * o.L, v, T(tm.eps));
    }
    weno_taps(P, tm, u, I, t, p, v);
    // the device copy of a WENO term stores 1/dx in `dx`
    return weno5_point<T>(v[0], v[1], v[2], v[3], v[4], T(tm.eps), T(tm.dx));
}

// Face value a(x_{I+1/2}, u~) * (D_inner u)_{I+1/2} of a nonlinear Laplacian term
// (nonlinear_laplacian.jl:28-103): u~ and x~ by the half-offset interpolation
// table, the inner derivative by the half-offset first-derivative table.
template <class T>
__device__ __noinline__ T nonlinlap_face(const DevProb<T>& P, const mol_term& tm, const T* u, const int* I, int Ih,
                            T t, const T* p) {
    const int f = tm.field, d = tm.dim, n = P.n[d];
    const bool per = (P.permask[f] >> d) & 1;
    int J[3] = {I[0], I[1], I[2]};
    // inner derivative at the half point
    const T du = apply_op_at(P, P.ops[tm.op2], u, f, d, I, Ih, n, t, p);
    if (tm.prog < 0) return du;
    // face program: a(x~, u~, p)
    const mol_op1d oip = P.ops[tm.op3];
    const TapSel sp = select_taps(oip, Ih, n, per);
    T r[MOL_MAX_REGS];
    T a = T(1);
    const int start = P.progs[2 * tm.prog], len = P.progs[2 * tm.prog + 1];
    for (int pc = start; pc < start + len; ++pc) {
        const mol_instr in = P.code[pc];
        T& R = r[in.dst];
        switch (in.op) {
            case MOL_OP_CONST: R = P.consts[in.imm]; break;
            case MOL_OP_PARAM: R = p[in.imm]; break;
            case MOL_OP_TIME: R = t; break;
            case MOL_OP_FIELD: {
                T acc = T(0);
                for (int k = 0; k < sp.cnt; ++k) {
                    int tp = sp.first + k;
                    if (per) tp = wrap_periodic(tp, n);
                    J[d] = tp;
                    const T v = load_pt(P, u, in.imm, J[0], J[1], J[2], t, p);
                    acc = k == 0 ? P.w[sp.woff] * v : fma(P.w[sp.woff + k], v, acc);
                }
                R = acc;
                break;
            }
            case MOL_OP_AUX: {
                // face array: extent n[d]+1 along d (index Ih), full-grid extents elsewhere
                R = P.aux[P.aux_off[tm.aux0 + in.imm] + face_index(P, d, Ih, I)];
                break;
            }
            case MOL_OP_ADD: R = r[in.a] + r[in.b]; break;
            case MOL_OP_SUB: R = r[in.a] - r[in.b]; break;
            case MOL_OP_MUL: R = r[in.a] * r[in.b]; break;
            case MOL_OP_DIV: R = r[in.a] / r[in.b]; break;
            case MOL_OP_NEG: R = -r[in.a]; break;
            case MOL_OP_POWI: R = powi(r[in.a], in.imm); break;
            case MOL_OP_POW: R = pow(r[in.a], r[in.b]); break;
            case MOL_OP_FN: R = apply_fn(in.imm, r[in.a]); break;
            case MOL_OP_CMP: R = apply_cmp(in.imm, r[in.a], r[in.b]); break;
            case MOL_OP_IFELSE: R = r[in.a] != T(0) ? r[in.b] : r[in.c]; break;
            case MOL_OP_OUT: a = r[in.a]; break;
            default: break;
        }
    }
    return a * du;
}

template <class T>
__device__ T apply_nonlinlap(const DevProb<T>& P, const mol_term& tm, const T* u, const int* I, T t, const T* p) {
    const int f = tm.field, d = tm.dim, n = P.n[d];
    const bool per = (P.permask[f] >> d) & 1;
    const mol_op1d oo = P.ops[tm.op];
    // outer half-offset stencil at II - 1 on a line clipped to n - 1 points; taps are half points
    const TapSel so = select_taps(oo, I[d] - 1, n - 1, per);
    T acc = T(0);
    bool started = false;
    for (int k = 0; k < so.cnt; ++k) {
        const T wo = P.w[so.woff + k];
        if (wo == T(0)) continue;  // zero outer weights drop out of the symbolic sum
        const int Ih = so.first + k;  // not wrapped: the face program wraps its own taps
        const T F = nonlinlap_face(P, tm, u, I, Ih, t, p);
        acc = started ? fma(wo, F, acc) : wo * F;
        started = true;
    }
    return acc;
}

template <class T>
__device__ __noinline__ T eval_term(const DevProb<T>& P, int k, const T* u, const int* I, T t, const T* p) {
    const mol_term tm = P.terms[k];
    switch (tm.kind) {
        case MOL_TERM_LINEAR: return apply_op(P, P.ops[tm.op], u, tm.field, tm.dim, I, t, p);
        case MOL_TERM_MIXED: return apply_mixed(P, tm, u, I, t, p);
        case MOL_TERM_WENO: return apply_weno(P, tm, u, I, t, p);
        case MOL_TERM_NONLINLAP: return apply_nonlinlap(P, tm, u, I, t, p);
        default: return T(0);
    }
}

// Full-grid index of interior cell `c` (flat, first dimension fastest).
template <class T>
__device__ __forceinline__ void cell_index(const DevProb<T>& P, long long c, int* I) {
    if (P.fastdiv) {
        const unsigned cc = (unsigned)c;
        const unsigned r = divq(cc, P.dm[0], P.ds[0]);
        const unsigned c2 = divq(r, P.dm[1], P.ds[1]);
        I[0] = (int)(cc - r * (unsigned)P.ni[0]) + 1 + P.lo[0];
        I[1] = (int)(r - c2 * (unsigned)P.ni[1]) + 1 + P.lo[1];
        I[2] = (int)c2 + 1 + P.lo[2];
        return;
    }
    const long long c0 = c % P.ni[0];
    const long long r = c / P.ni[0];
    const long long c1 = r % P.ni[1];
    const long long c2 = r / P.ni[1];
    I[0] = (int)c0 + 1 + P.lo[0];
    I[1] = (int)c1 + 1 + P.lo[1];
    I[2] = (int)c2 + 1 + P.lo[2];
}

// The cell program: one OUT per field.  `out` receives du for every field.
template <class T>
__device__ __noinline__ void eval_cell(const DevProb<T>& P, const T* u, long long c, const int* I, T t, const T* p, T* out) {
    T r[MOL_MAX_REGS];
    const int start = P.progs[2 * P.cell_prog], len = P.progs[2 * P.cell_prog + 1];
    for (int pc = start; pc < start + len; ++pc) {
        const mol_instr in = P.code[pc];
        T& R = r[in.dst];
        switch (in.op) {
            case MOL_OP_CONST: R = P.consts[in.imm]; break;
            case MOL_OP_PARAM: R = p[in.imm]; break;
            case MOL_OP_FIELD: R = u[(long long)in.imm * P.ncell + c]; break;
            case MOL_OP_AUX: R = P.aux[P.aux_off[in.imm] + c]; break;
            case MOL_OP_COORD: R = P.coords[in.imm][I[in.imm] - 1]; break;
            case MOL_OP_TIME: R = t; break;
            case MOL_OP_TERM: R = eval_term(P, in.imm, u, I, t, p); break;
            case MOL_OP_UPWIND: {
                // rhs term kappa*Dx^d(u) is (-kappa)*Dx^d(u) on the cardinalised lhs; the reference
                // takes the backward (windmap[2]) stencil when that coefficient is > 0.
                const T kap = r[in.a];
                R = kap < T(0) ? kap * eval_term(P, in.b, u, I, t, p) : kap * eval_term(P, in.c, u, I, t, p);
                break;
            }
            case MOL_OP_ADD: R = r[in.a] + r[in.b]; break;
            case MOL_OP_SUB: R = r[in.a] - r[in.b]; break;
            case MOL_OP_MUL: R = r[in.a] * r[in.b]; break;
            case MOL_OP_DIV: R = r[in.a] / r[in.b]; break;
            case MOL_OP_NEG: R = -r[in.a]; break;
            case MOL_OP_POWI: R = powi(r[in.a], in.imm); break;
            case MOL_OP_POW: R = pow(r[in.a], r[in.b]); break;
            case MOL_OP_FN: R = apply_fn(in.imm, r[in.a]); break;
            case MOL_OP_CMP: R = apply_cmp(in.imm, r[in.a], r[in.b]); break;
            case MOL_OP_IFELSE: R = r[in.a] != T(0) ? r[in.b] : r[in.c]; break;
            case MOL_OP_OUT: out[in.imm] = r[in.a]; break;
            default: break;
        }
    }
}

}  // namespace mol
