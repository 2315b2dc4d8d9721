// Kernel templates of the hot path.  `G` supplies the per-cell right-hand side
// (`G::cell`) and its vector-Jacobian product (`G::cell_vjp`): either the
// register-machine interpreter (always built) or the straight-line code that
// the library generates for a plan and compiles with NVRTC.
#pragma once

#include "mol_device.cuh"
#include "mol_vjp.cuh"

namespace mol {

constexpr int kThreads = 256;

// Minimum resident CTAs per SM requested from the register allocator for the kernels that
// evaluate the right-hand side (set for generated modules, MOL_JIT_MIN_BLOCKS).
#ifndef MOL_BATCH_MIN_BLOCKS
// ensemble kernels: CTAs of kThreads per SM the register budget must allow.  Uncapped the tiled
// kernel took 134 registers and the autotuner fell back to one CTA per instance (48 s -> 79 s
// for the 4096 members' 1000 steps); at 2 (128 registers, no spills) 1024 members' 200 steps
// took 2.65 s, at 3 (85 registers, some spills, 24 warps per SM) 2.42 s
#define MOL_BATCH_MIN_BLOCKS 3
#endif
#ifndef MOL_MIN_BLOCKS
#define MOL_MIN_BLOCKS 1
#endif
// The face pass moves ~7 bytes per FP64 instruction: it needs more warps in flight than the
// stage kernels, so its register budget allows more resident CTAs (set for generated modules).
#ifndef MOL_FACE_MIN_BLOCKS
#define MOL_FACE_MIN_BLOCKS MOL_MIN_BLOCKS
#endif
// The vector-Jacobian product holds the forward values and partials of a whole cell: at the
// stage kernels' 80-register budget it spilled 2.2 KB per thread (ptxas), so it gets its own.
#ifndef MOL_VJP_MIN_BLOCKS
#define MOL_VJP_MIN_BLOCKS MOL_MIN_BLOCKS
#endif

// Correctly rounded x/3 with one multiply and two FMAs (Markstein's theorem:
// with c = RN(1/3) and q0 within an ulp of x/3, q0 + (x - 3 q0) c rounds to
// RN(x/3)); replaces the FP64 division of SSPRK33's last stage.
__device__ __forceinline__ double div3m(double x) {
    const double c = 0.33333333333333331483;  // RN(1/3)
    const double q0 = x * c;
    const double r = fma(-q0, 3.0, x);
    return fma(r, c, q0);
}
__device__ __forceinline__ float div3m(float x) { return x / 3.0f; }

// Finite test on the exponent bits (integer instructions: no FP64 pipe time).  The last
// SSPRK33 stage ORs it over its outputs, the counterpart of OrdinaryDiffEq's unstable_check
// (any NaN in u ends the solve): a NaN or Inf anywhere in a stage reaches the step's result.
__device__ __forceinline__ bool nonfinite_bits(double x) {
    return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
}
__device__ __forceinline__ bool nonfinite_bits(float x) {
    return ((unsigned)__float_as_int(x) & 0x7f800000u) == 0x7f800000u;
}

// One flag per warp that saw a non-finite value (every lane of the warp must call it).
__device__ __forceinline__ void flag_nonfinite(bool bad, int* flag) {
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

struct InterpCell {
    static constexpr int kFields = 0;  // field count known only at run time
    static constexpr int kFaceTerms = 0;  // the interpreter evaluates every face in the cell
    static constexpr int kCoefArrays = 0; // and has no coefficient stencils
    template <class T>
    static __device__ __forceinline__ void faces(const DevProb<T>&, const T*, long long, const int*, T, const T*, T*) {}
    template <class T>
    struct Uniform {};
    template <class T>
    static __device__ __forceinline__ void uniform(const DevProb<T>&, T, const T*, Uniform<T>&) {}
    template <class T>
    static __device__ __forceinline__ void cell(const DevProb<T>& P, const T* __restrict__ u, long long c,
                                                const int* I, T t, const T* __restrict__ p, const Uniform<T>&,
                                                T* out) {
        eval_cell(P, u, c, I, t, p, out);
    }
};

// Fields per cell: a compile-time constant for generated cells (so per-field loops unroll
// and the per-cell output arrays stay in registers), the descriptor's count otherwise.
template <class G, class T>
__device__ __forceinline__ int nfields_of(const DevProb<T>& P) {
    return G::kFields > 0 ? G::kFields : P.nfields;
}

template <class T, class G>
__global__ void __launch_bounds__(kThreads, MOL_MIN_BLOCKS) k_rhs_t(const __grid_constant__ DevProb<T> P, const T* __restrict__ u, T* __restrict__ du,
                                                    const T* __restrict__ p, double t) {
    T out[MOL_MAX_FIELDS];
    typename G::template Uniform<T> U;
    G::uniform(P, T(t), p, U);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < P.ncell;
         c += (long long)gridDim.x * blockDim.x) {
        int I[3];
        cell_index(P, c, I);
        G::cell(P, u, c, I, T(t), p, U, out);
        #pragma unroll
        for (int f = 0; f < nfields_of<G>(P); ++f) du[(long long)f * P.ncell + c] = out[f];
    }
}

// The face pass: for every cell, the left face (half point I - 1/2 along the term's
// dimension) of each nonlinear-Laplacian term, so the cell kernel that follows reads a face
// computed once instead of evaluating it for both cells that share it.  The time is
// S->t (tfix NaN) or tfix, plus toff, exactly as the stage kernel forms its stage time.
template <class T, class G>
__global__ void __launch_bounds__(kThreads, MOL_FACE_MIN_BLOCKS) k_faces_t(const __grid_constant__ DevProb<T> P,
                                                                      const T* __restrict__ u,
                                                                      const T* __restrict__ p, const SolverState* S,
                                                                      double toff, double tfix, T* __restrict__ faces) {
    constexpr int NQ = G::kFaceTerms > 0 ? G::kFaceTerms : 1;
    if (G::kFaceTerms == 0) return;
    const double t0 = (tfix == tfix) ? tfix : S->t;
    const double t = toff == 0.0 ? t0 : t0 + toff;
    T out[NQ];
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < P.ncell;
         c += (long long)gridDim.x * blockDim.x) {
        int I[3];
        cell_index(P, c, I);
        G::faces(P, u, c, I, T(t), p, out);
#pragma unroll
        for (int q = 0; q < NQ; ++q) faces[(long long)q * P.fstride + c] = out[q];
    }
}

// Coefficient stencils: the per-cell coefficient arrays of the generated cell's variable
// groups ([array][cell], FP64, and an FP32 copy for the Float32-state kernels when cw32 is
// set), computed once at plan creation from the face programs of coordinate-dependent
// nonlinear Laplacians.
template <class G>
__global__ void __launch_bounds__(kThreads) k_coef_t(const __grid_constant__ DevProb<double> P, double* __restrict__ cw,
                                                     float* __restrict__ cw32) {
    constexpr int NA = G::kCoefArrays > 0 ? G::kCoefArrays : 1;
    if (G::kCoefArrays == 0) return;
    double out[NA];
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < P.ncell;
         c += (long long)gridDim.x * blockDim.x) {
        int I[3];
        cell_index(P, c, I);
        G::coefs(P, c, I, out);
#pragma unroll
        for (int q = 0; q < NA; ++q) {
            cw[(long long)q * P.ncell + c] = out[q];
            if (cw32) cw32[(long long)q * P.ncell + c] = (float)out[q];
        }
    }
}

// SSPRK33 stage epilogue with OrdinaryDiffEq's evaluation order:
//   1: u1 = u0 + dt k     2: u2 = (3 u0 + u1 + dt k)/4     3: u = (u0 + 2 u2 + 2 dt k)/3
// u0 + 2 u2 is written as fma(2, u2, u0): 2 u2 is exact, so it is the same correctly rounded
// sum, in one instruction whatever the compiler's contraction choices.
template <class T, int STAGE>
__device__ __forceinline__ T ssprk_combine(T u0, T uin, T k, T dt, T dt2) {
    if (STAGE == 1) return u0 + dt * k;
    if (STAGE == 2) return ((T(3) * u0 + uin) + dt * k) * T(0.25);
    return div3m(fma(dt2, k, fma(T(2), uin, u0)));
}

__device__ __forceinline__ void last_block_advance(SolverState* S, double t_new) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned v = atomicAdd(&S->blocks_done, 1u);
        if (v == gridDim.x - 1) {
            S->t = t_new;
            S->blocks_done = 0;
            __threadfence();
        }
    }
}

// `tfix` (when not NaN) is the step's start time, used instead of S->t and leaving S alone:
// the adjoint recomputes single stages at known times without touching the solver state.
// Cells [cbeg, cend) are processed (stage 1 runs in slabs while the state arrives from the
// host; every other launch covers all cells).  Stages 1 and 2 take the step in `dts`, stage 3
// takes 2 dt, the coefficient of its combination, so that the cell loop reads it from the
// kernel's parameters instead of forming 2 dt again per cell.
template <class T, class G, int STAGE>
__global__ void __launch_bounds__(kThreads, MOL_MIN_BLOCKS) k_ssprk_t(const __grid_constant__ DevProb<T> P, const T* __restrict__ uin, const T* u0, T* uout,
                                                      const T* __restrict__ p, SolverState* S, double dts,
                                                      double tfix, long long cbeg, long long cend) {
    const double dt = STAGE == 3 ? 0.5 * dts : dts;
    const bool from_state = !(tfix == tfix);
    const double t0 = from_state ? S->t : tfix;
    const double ts = STAGE == 1 ? t0 : (STAGE == 2 ? t0 + dt : t0 + dt / 2);
    T out[MOL_MAX_FIELDS];
    typename G::template Uniform<T> U;
    G::uniform(P, T(ts), p, U);
    bool bad = false;
    for (long long c = cbeg + blockIdx.x * (long long)blockDim.x + threadIdx.x; c < cend;
         c += (long long)gridDim.x * blockDim.x) {
        int I[3];
        cell_index(P, c, I);
        G::cell(P, uin, c, I, T(ts), p, U, out);
        #pragma unroll
        for (int f = 0; f < nfields_of<G>(P); ++f) {
            const long long g = (long long)f * P.ncell + c;
            const T r = ssprk_combine<T, STAGE>(u0[g], uin[g], out[f], T(dt), T(dts));
            if (STAGE == 3) bad |= nonfinite_bits(r);
            uout[g] = r;
        }
    }
    if (STAGE == 3) flag_nonfinite(bad, &S->nonfinite);
    if (STAGE == 3 && from_state) last_block_advance(S, t0 + dt);
}

// Vector-Jacobian product of the RHS: lam_u += scale * (df/du)^T lam, lam_p and lam_aux likewise.
// Parameter adjoints are reduced per block before one atomic per block and parameter.
// The adjoint seed of a VJP launch, read cell by cell: v = sum_k a[k] x[k] (null x[k]
// skipped), seed = scale * v.  When `upd` is set, v is also written there, and the
// `zero` arrays are cleared, all at the cell being processed (so one of the x[k] may be
// updated in place).  This folds the linear combinations of the reverse RK sweep into
// the VJP launches that read them.
template <class T>
struct VjpSeed {
    const T* x[4];
    T a[4];
    T* upd;
    T* zero[3];
};

template <class T, class G, int NP>
__global__ void __launch_bounds__(kThreads, MOL_VJP_MIN_BLOCKS) k_vjp_t(const __grid_constant__ DevProb<T> P,
                                                                    const VjpSeed<T> in, T scale,
                                                                    const T* __restrict__ u, const T* __restrict__ p,
                                                                    double t, T* lam_u, T* lam_p, T* lam_aux) {
    T lp[NP > 0 ? NP : 1];
#pragma unroll
    for (int k = 0; k < (NP > 0 ? NP : 1); ++k) lp[k] = T(0);
    T seed[MOL_MAX_FIELDS];
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < P.ncell;
         c += (long long)gridDim.x * blockDim.x) {
        int I[3];
        cell_index(P, c, I);
        #pragma unroll
        for (int f = 0; f < nfields_of<G>(P); ++f) {
            const long long q = (long long)f * P.ncell + c;
            T v = in.a[0] * in.x[0][q];
#pragma unroll
            for (int k = 1; k < 4; ++k)
                if (in.x[k]) v += in.a[k] * in.x[k][q];
            if (in.upd) in.upd[q] = v;
#pragma unroll
            for (int k = 0; k < 3; ++k)
                if (in.zero[k]) in.zero[k][q] = T(0);
            seed[f] = scale * v;
        }
        G::cell_vjp(P, u, c, I, T(t), p, seed, lam_u, lp, lam_aux);
    }
    if (NP > 0 && lam_p) {
        __shared__ T red[kThreads / 32];
        for (int k = 0; k < NP; ++k) {
            T v = lp[k];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
            __syncthreads();
            if (threadIdx.x == 0) {
                T s = T(0);
                for (int w = 0; w < (int)(blockDim.x / 32); ++w) s += red[w];
                atomicAdd(lam_p + k, s);
            }
            __syncthreads();
        }
    }
}

// One persistent launch for a whole ensemble: each CTA takes the next instance
// (largest first, dynamic via an atomic ticket) and integrates it for `nsteps`
// SSPRK33 steps, synchronising only its own threads between stages.
template <class T, class G>
__global__ void __launch_bounds__(kThreads, MOL_BATCH_MIN_BLOCKS) k_batch_ssprk_t(const DevProb<T>* __restrict__ probs,
                                                            const long long* __restrict__ off,
                                                            const int* __restrict__ order, int ninst, T* U, T* U1,
                                                            T* U2, const T* const* __restrict__ params,
                                                            const double* __restrict__ dts, double t0,
                                                            long long nsteps, unsigned* ticket, int* nonfinite) {
    __shared__ int slot;
    T out[MOL_MAX_FIELDS];
    typename G::template Uniform<T> UN;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) slot = (int)atomicAdd(ticket, 1u);
        __syncthreads();
        if (slot >= ninst) return;
        const int i = order[slot];
        const DevProb<T>& P = probs[i];
        T* u = U + off[i];
        T* u1 = U1 + off[i];
        T* u2 = U2 + off[i];
        const T* p = params[i];
        const double dt = dts[i];
        const long long nc = P.ncell;
        double t = t0;
        for (long long s = 0; s < nsteps; ++s) {
            G::uniform(P, T(t), p, UN);
            for (long long c = threadIdx.x; c < nc; c += blockDim.x) {
                int I[3];
                cell_index(P, c, I);
                G::cell(P, u, c, I, T(t), p, UN, out);
                #pragma unroll
                for (int f = 0; f < nfields_of<G>(P); ++f) {
                    const long long g = (long long)f * nc + c;
                    u1[g] = ssprk_combine<T, 1>(u[g], u[g], out[f], T(dt), T(2 * dt));
                }
            }
            __syncthreads();
            G::uniform(P, T(t + dt), p, UN);
            for (long long c = threadIdx.x; c < nc; c += blockDim.x) {
                int I[3];
                cell_index(P, c, I);
                G::cell(P, u1, c, I, T(t + dt), p, UN, out);
                #pragma unroll
                for (int f = 0; f < nfields_of<G>(P); ++f) {
                    const long long g = (long long)f * nc + c;
                    u2[g] = ssprk_combine<T, 2>(u[g], u1[g], out[f], T(dt), T(2 * dt));
                }
            }
            __syncthreads();
            G::uniform(P, T(t + dt / 2), p, UN);
            bool bad = false;
            for (long long c = threadIdx.x; c < nc; c += blockDim.x) {
                int I[3];
                cell_index(P, c, I);
                G::cell(P, u2, c, I, T(t + dt / 2), p, UN, out);
                #pragma unroll
                for (int f = 0; f < nfields_of<G>(P); ++f) {
                    const long long g = (long long)f * nc + c;
                    const T r = ssprk_combine<T, 3>(u[g], u2[g], out[f], T(dt), T(2 * dt));
                    bad |= nonfinite_bits(r);
                    u[g] = r;
                }
            }
            flag_nonfinite(bad, nonfinite);
            __syncthreads();
            t = t + dt;
        }
    }
}


// ---------------------------------------------------------------------------
// Tiled ensemble kernel.  The unit of work is one tile (tile_cells consecutive
// cells) of one stage of one instance, so a large instance spreads over many
// CTAs while small ones still take a single tile.  Work items are handed out by
// one 64-bit ticket in round-major order (round r = 3 * step + stage; within a
// round, instances largest first, then their tiles).  Before a tile of round r
// runs, every tile of rounds < r of the same instance must be done: a
// per-instance counter of finished tiles (release-add after the tile, acquire
// poll before it) carries that dependency.  A CTA only ever waits for items
// with smaller tickets, which were handed to CTAs that are already running, so
// the lowest unfinished ticket can always proceed.  Each wait is bounded: past
// MOL_BATCH_SPIN_LIMIT polls it sets the shared status word and every CTA
// leaves at its next poll or ticket.

#define MOL_BATCH_SPIN_LIMIT (1ll << 25)

struct BatchSync {
    unsigned long long* ticket;   // next work item
    unsigned long long* done;     // [instance] tiles finished, all rounds so far
    int* status;                  // 0 ok, 1 a wait ran out of budget
    long long spin_limit;         // polls before a wait gives up (MOL_BATCH_SPIN_LIMIT by default)
    int* nonfinite;               // set when a step's result holds a NaN or Inf (sticky)
};

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Tile g of a round: its instance (slot order already resolved), its index within the
// instance and the instance's tile count.
struct TileRef {
    int inst, tile, ntiles, pad;
};

// One SSPRK33 stage of cells [cb, ce) of an instance (the CTA's threads stride over them);
// returns whether a last-stage result of this thread was NaN or Inf.
template <class T, class G, int STAGE>
__device__ __forceinline__ bool batch_cells(const DevProb<T>& P, const T* __restrict__ uin, const T* u0, T* uout,
                                            const T* __restrict__ p, double ts, double dt, long long cb,
                                            long long ce, const typename G::template Uniform<T>& UN) {
    T out[MOL_MAX_FIELDS];
    bool bad = false;
    const long long nc = P.ncell;
    for (long long c = cb + threadIdx.x; c < ce; c += blockDim.x) {
        int I[3];
        cell_index(P, c, I);
        G::cell(P, uin, c, I, T(ts), p, UN, out);
#pragma unroll
        for (int f = 0; f < nfields_of<G>(P); ++f) {
            const long long q = (long long)f * nc + c;
            const T r = ssprk_combine<T, STAGE>(u0[q], uin[q], out[f], T(dt), T(2 * dt));
            if (STAGE == 3) bad |= nonfinite_bits(r);
            uout[q] = r;
        }
    }
    return bad;
}

// The same stage with the nonlinear-Laplacian faces computed once: cells [cb, ce) go in chunks;
// for each chunk the CTA first writes the left face of every cell the chunk's cells read
// (the chunk plus one line of the slowest face dimension) into a shared-memory window of W
// cells per face term, then runs the cells on a copy of the problem view (sP, in shared
// memory) whose faces point at the window.  Each face is then evaluated once per chunk
// instead of once for each of the two cells that share it; the values are the ones the
// cells would compute themselves (the same generated code), so results are unchanged.
// Instances whose face line does not fit the window run without it.
template <class T, class G, int STAGE>
__device__ bool batch_cells_faces(const DevProb<T>& Pg, DevProb<T>& sP, T* win, long long W, const T* __restrict__ uin,
                                  const T* u0, T* uout, const T* __restrict__ p, double ts, double dt, long long cb,
                                  long long ce, const typename G::template Uniform<T>& UN) {
    constexpr int NQ = G::kFaceTerms > 0 ? G::kFaceTerms : 1;
    const long long nc = Pg.ncell;
    const long long line = gstride(Pg, Pg.ndim - 1);   // cells between neighbours along the slowest dimension
    const long long chunk = W - line;
    if (G::kFaceTerms == 0 || W <= 0 || chunk < (long long)blockDim.x)
        return batch_cells<T, G, STAGE>(Pg, uin, u0, uout, p, ts, dt, cb, ce, UN);
    bool bad = false;
    for (long long a = cb; a < ce; a += chunk) {
        const long long b = min(ce, a + chunk);
        const long long fe = min(nc, b + line);
        for (long long c = a + threadIdx.x; c < fe; c += blockDim.x) {
            int I[3];
            cell_index(Pg, c, I);
            T fo[NQ];
            G::faces(Pg, uin, c, I, T(ts), p, fo);
#pragma unroll
            for (int q = 0; q < NQ; ++q) win[(long long)q * W + (c - a)] = fo[q];
        }
        if (threadIdx.x == 0) {
            sP.faces = win - a;   // faces[q * W + c] is the window's entry of cell c, for c in [a, fe)
            sP.fbeg = a;
            sP.fend = fe;
        }
        __syncthreads();
        bad |= batch_cells<T, G, STAGE>(sP, uin, u0, uout, p, ts, dt, a, b, UN);
        __syncthreads();
    }
    return bad;
}

template <class T, class G>
__global__ void __launch_bounds__(kThreads, MOL_BATCH_MIN_BLOCKS) k_batch_tiles_t(const DevProb<T>* __restrict__ probs,
                                                            const long long* __restrict__ off,
                                                            const TileRef* __restrict__ tiles,
                                                            long long ntiles, int tile_cells, T* U, T* U1, T* U2,
                                                            const T* const* __restrict__ params,
                                                            const double* __restrict__ dts, double t0,
                                                            long long nsteps, BatchSync sync, long long face_window) {
    __shared__ long long s_item;
    __shared__ TileRef s_ref;
    __shared__ int s_ok;
    // the face window (dynamic shared memory, face_window cells per face term) and the
    // problem view that points at it
    extern __shared__ __align__(16) unsigned char mol_batch_smem[];
    __shared__ DevProb<T> sP;
    T* win = reinterpret_cast<T*>(mol_batch_smem);
    const long long nitems = 3 * nsteps * ntiles;
    typename G::template Uniform<T> UN;
    // thread 0 takes the next ticket while the CTA works on the current tile; the held ticket
    // is larger than the one being worked on, so the lowest unfinished unit still always runs
    long long next = 0;
    if (threadIdx.x == 0) next = *(volatile int*)sync.status ? nitems : (long long)atomicAdd(sync.ticket, 1ull);
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const long long item = next;
            s_item = item;
            int ok = 1;
            if (item < nitems) {
                const long long r = item / ntiles;
                const TileRef ref = tiles[item - r * ntiles];
                s_ref = ref;
                const unsigned long long need = (unsigned long long)(r * ref.ntiles);
                long long polls = 0;
                while (ld_acquire_u64(sync.done + ref.inst) < need) {
                    if (*(volatile int*)sync.status != 0) {
                        ok = 0;
                        break;
                    }
                    if (++polls > sync.spin_limit) {
                        atomicExch(sync.status, 1);
                        ok = 0;
                        break;
                    }
                    __nanosleep(64);
                }
                if (ok) next = *(volatile int*)sync.status ? nitems : (long long)atomicAdd(sync.ticket, 1ull);
            }
            s_ok = ok;
        }
        __syncthreads();
        const long long item = s_item;
        if (item >= nitems || !s_ok) return;
        const long long r = item / ntiles;
        const int i = s_ref.inst;
        const long long j = s_ref.tile;
        const DevProb<T>& P = probs[i];
        T* u = U + off[i];
        T* u1 = U1 + off[i];
        T* u2 = U2 + off[i];
        const T* p = params[i];
        const double dt = dts[i];
        const long long nc = P.ncell;
        const int stage = (int)(r % 3);
        const double t = t0 + (double)(r / 3) * dt;
        const long long c_beg = j * (long long)tile_cells;
        const long long c_end = min(nc, (j + 1) * (long long)tile_cells);
        if (G::kFaceTerms > 0 && face_window > 0 && threadIdx.x == 0) {
            sP = P;
            sP.fstride = face_window;
        }
        if (stage == 0) {
            G::uniform(P, T(t), p, UN);
            batch_cells_faces<T, G, 1>(P, sP, win, face_window, u, u, u1, p, t, dt, c_beg, c_end, UN);
        } else if (stage == 1) {
            G::uniform(P, T(t + dt), p, UN);
            batch_cells_faces<T, G, 2>(P, sP, win, face_window, u1, u, u2, p, t + dt, dt, c_beg, c_end, UN);
        } else {
            G::uniform(P, T(t + dt / 2), p, UN);
            const bool bad =
                batch_cells_faces<T, G, 3>(P, sP, win, face_window, u2, u, u, p, t + dt / 2, dt, c_beg, c_end, UN);
            flag_nonfinite(bad, sync.nonfinite);
        }
        __syncthreads();
        if (threadIdx.x == 0) red_release_add_u64(sync.done + i, 1ull);
    }
}

// Tsitouras (2011) nodes c_i of the 5(4) pair OrdinaryDiffEq's Tsit5 implements.
__device__ __forceinline__ double tsit_c(int i) {
    switch (i) {
        case 2: return 0.161;
        case 3: return 0.327;
        case 4: return 0.9;
        case 5: return 0.9800255409045097;
        default: return 1.0;
    }
}

// Row updates of the controller's dt-scaled tableau (Tsitouras 2011 a_ij and btilde_j); one thread.
__device__ __forceinline__ void tsit_scale(SolverState* S) {
    const double A[8][8] = {
        {0}, {0},
        {0, 0.161},
        {0, -0.008480655492356989, 0.335480655492357},
        {0, 2.897153057105493, -6.359448489975075, 4.3622954328695815},
        {0, 5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525},
        {0, 5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383},
        {0, 0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081,
         2.324710524099774}};
    const double B[8] = {0, -0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                         -0.1447110071732629, 0.5823571654525552, -0.45808210592918697, 0.015151515151515152};
    const double dt = S->dt;
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j) S->dta[i][j] = dt * A[i][j];
    for (int j = 0; j < 8; ++j) S->dtb[j] = dt * B[j];
}

// Stage i (2..7) on cells c_beg, c_beg + c_step, ...: k_i = f(y_i, t), and y_{i+1} = u +
// sum_j (dt a_{i+1,j}) k_j, or at stage 7 the scaled error sum_j (dt btilde_j) k_j, whose
// squared norm terms are returned.
template <class T, class G>
__device__ __forceinline__ double tsit_stage_cells(const DevProb<T>& P, int stage, const T* __restrict__ y, T* ynext,
                                                   const T* __restrict__ u, T* const* k, const T* __restrict__ p,
                                                   const SolverState* S, double t, long long c_beg, long long c_step) {
    T out[MOL_MAX_FIELDS];
    double errsq = 0.0;
    const double abstol = S->abstol, reltol = S->reltol;
    typename G::template Uniform<T> U;
    G::uniform(P, T(t), p, U);
    for (long long c = c_beg; c < P.ncell; c += c_step) {
        int I[3];
        cell_index(P, c, I);
        G::cell(P, y, c, I, T(t), p, U, out);
        #pragma unroll
        for (int f = 0; f < nfields_of<G>(P); ++f) {
            const long long g = (long long)f * P.ncell + c;
            k[stage - 1][g] = out[f];
            if (stage < 7) {
                T acc = u[g];
                for (int j = 1; j <= stage; ++j) {
                    const T kj = j == stage ? out[f] : k[j - 1][g];
                    acc = fma(T(S->dta[stage + 1][j]), kj, acc);
                }
                ynext[g] = acc;
            } else {
                T e = T(0);
                for (int j = 1; j <= 7; ++j) {
                    const T kj = j == 7 ? out[f] : k[j - 1][g];
                    e = fma(T(S->dtb[j]), kj, e);
                }
                const double sc = abstol + fmax(fabs((double)u[g]), fabs((double)y[g])) * reltol;
                const double r = (double)e / sc;
                errsq = fma(r, r, errsq);
            }
        }
    }
    return errsq;
}

// The PI step-size controller (OrdinaryDiffEq's for Tsit5) given the error norm's sum of squares
// over N values; one thread.
__device__ __forceinline__ void tsit_control(SolverState* S, double s, double N, double qold_pow = -1.0) {
    const double EEst = sqrt(s / N);
    S->EEst = EEst;
    S->nf += 6;
    S->iter += 1;
    if (!isfinite(EEst)) {
        S->status = MOL_ERR_NONFINITE;
        S->done = 1;
        S->accepted = 0;
        return;
    }
    // PI controller (beta1 = 7/50, beta2 = 2/25, qmin = 1/5, qmax = 10, gamma = 9/10)
    const double beta1 = 0.14, beta2 = 0.08, qmin = 0.2, qmax = 10.0, gamma = 0.9, qoldinit = 1e-4;
    const double q11 = pow(EEst, beta1);
    const double dt = S->dt;
    double dtnew;
    if (EEst <= 1.0) {
        double q = q11 / (qold_pow >= 0.0 ? qold_pow : pow(S->qold, beta2));
        q = fmax(1.0 / qmax, fmin(1.0 / qmin, q / gamma));
        S->t = S->t + dt;
        S->qold = fmax(EEst, qoldinit);
        dtnew = dt / q;
        S->naccept += 1;
        S->accepted = 1;
        if (S->t >= S->t1) S->done = 1;
    } else {
        const double q = fmin(1.0 / qmin, q11 / gamma);
        dtnew = dt / q;
        S->nreject += 1;
        S->accepted = 0;
    }
    if (!S->done) {
        if (S->t + dtnew > S->t1) dtnew = S->t1 - S->t;
        if (!(dtnew > S->dtmin) && S->t < S->t1) {
            S->status = MOL_ERR_DTMIN;
            S->done = 1;
        }
        if (S->iter >= S->maxiters) {
            S->status = MOL_ERR_MAXITERS;
            S->done = 1;
        }
    }
    S->dt = dtnew;
    __threadfence();
}

// Stage i (2..7) over the grid; at stage 7 the last block to finish reduces the error norm
// deterministically (block order) and runs the controller.
template <class T, class G>
__global__ void __launch_bounds__(kThreads, MOL_MIN_BLOCKS) k_tsit_stage_t(const __grid_constant__ DevProb<T> P, int stage, const T* __restrict__ y,
                                                           T* ynext, const T* __restrict__ u, T* const* k,
                                                           const T* __restrict__ p, SolverState* S,
                                                           double* partials) {
    if (S->done) return;
    const double t = S->t + tsit_c(stage) * S->dt;
    double errsq = tsit_stage_cells<T, G>(P, stage, y, ynext, u, k, p, S, t,
                                          blockIdx.x * (long long)blockDim.x + threadIdx.x,
                                          (long long)gridDim.x * blockDim.x);
    if (stage < 7) return;
    __shared__ double red[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) errsq += __shfl_down_sync(0xffffffffu, errsq, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = errsq;
    __syncthreads();
    __shared__ bool last;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) s += red[w];
        partials[blockIdx.x] = s;
        __threadfence();
        const unsigned v = atomicAdd(&S->blocks_done, 1u);
        last = (v == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double s = 0.0;
    for (unsigned b = 0; b < gridDim.x; ++b) s += ((volatile double*)partials)[b];
    S->blocks_done = 0;
    tsit_control(S, s, (double)P.ncell * P.nfields);
}

// Tsit5 for small problems: one CTA owns the whole state and runs up to `attempts` attempts
// (stages 2..7, the error norm, the controller and the commit) in one launch, with block
// barriers between the phases instead of kernel boundaries; the host checks S->done between
// launches.  With `smem` set (dynamic shared memory of 10 state arrays) the state, the seven
// stage values and the two stage inputs live in shared memory for the launch, and the solver
// state is worked on in a shared copy.  For a few hundred unknowns the seven launches of an
// attempt, and its loads from L2, cost more than its arithmetic.  y2 must be formed before
// the first launch (k_tsit_commit, first).
template <class T, class G>
__global__ void __launch_bounds__(kThreads) k_tsit_small_t(const __grid_constant__ DevProb<T> P, T* u,
                                                          T* const* k, T* yb0, T* yb1, const T* __restrict__ p,
                                                          SolverState* S, int attempts, int smem) {
    extern __shared__ __align__(16) unsigned char tsit_smem[];
    __shared__ SolverState Ss;
    __shared__ double red[kThreads / 32];
    __shared__ double qpow;
    __shared__ int stop;
    const long long n = P.ncell * nfields_of<G>(P);
    T* su = u;
    T* sy0 = yb0;
    T* sy1 = yb1;
    T* sk[7];
    for (int j = 0; j < 7; ++j) sk[j] = k[j];
    if (smem) {
        T* base = (T*)tsit_smem;
        su = base;
        sy0 = base + n;
        sy1 = base + 2 * n;
        for (int j = 0; j < 7; ++j) sk[j] = base + (3 + j) * n;
        for (long long g = threadIdx.x; g < n; g += blockDim.x) {
            su[g] = u[g];
            sy0[g] = yb0[g];
            sk[0][g] = k[0][g];
        }
    }
    if (threadIdx.x == 0) Ss = *S;
    __syncthreads();
    const double beta2 = 0.08;
    for (int a = 0; a < attempts; ++a) {
        if (threadIdx.x == 0) stop = Ss.done;
        // the controller's pow(qold, beta2) on another warp, off the critical path
        if (threadIdx.x == 32 || (blockDim.x <= 32 && threadIdx.x == 0)) qpow = pow(Ss.qold, beta2);
        __syncthreads();
        if (stop) break;
        double errsq = 0.0;
        for (int stage = 2; stage <= 7; ++stage) {
            const T* yin = (stage % 2 == 0) ? sy0 : sy1;
            T* yout = (stage % 2 == 0) ? sy1 : sy0;
            const double t = Ss.t + tsit_c(stage) * Ss.dt;
            const double e = tsit_stage_cells<T, G>(P, stage, yin, yout, su, sk, p, &Ss, t, threadIdx.x, blockDim.x);
            if (stage == 7) errsq = e;
            __syncthreads();
        }
        for (int o = 16; o > 0; o >>= 1) errsq += __shfl_down_sync(0xffffffffu, errsq, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = errsq;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < (int)((blockDim.x + 31) / 32); ++w) s += red[w];
            tsit_control(&Ss, s, (double)n, qpow);
        }
        __syncthreads();
        // commit an accepted step (u <- y7, k1 <- k7) and form y2 = u + dt a21 k1 for the next
        const bool acc = Ss.accepted, done = Ss.done;
        const T a21 = T(Ss.dt * 0.161);
        for (long long g = threadIdx.x; g < n; g += blockDim.x) {
            T uu, kk;
            if (acc) {
                uu = sy1[g];
                kk = sk[6][g];
                su[g] = uu;
                sk[0][g] = kk;
            } else {
                uu = su[g];
                kk = sk[0][g];
            }
            if (!done) sy0[g] = fma(a21, kk, uu);
        }
        __syncthreads();
        if (threadIdx.x == 0) tsit_scale(&Ss);
        __syncthreads();
    }
    if (smem) {
        for (long long g = threadIdx.x; g < n; g += blockDim.x) {
            u[g] = su[g];
            yb0[g] = sy0[g];
            k[0][g] = sk[0][g];
        }
    }
    if (threadIdx.x == 0) {
        *S = Ss;
        __threadfence();
    }
}

}  // namespace mol
