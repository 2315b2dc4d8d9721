// libmolgpu: plan creation, f!(du,u,p,t), fixed-step SSPRK33 and adaptive Tsit5.
//
// Replaces, at runtime, the ModelingToolkit-compiled ODEFunction that
// MethodOfLines.jl builds in src/MOL_discretization.jl:171-201 and the
// OrdinaryDiffEq steppers that call it (benchmark/weno/suite.jl:283-295).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include <string>
#include <vector>

#include "mol_device.cuh"
#include "mol_kernels.cuh"
#include "mol_plan.h"

namespace mol {

std::atomic<long long> g_launches{0};

int set_err(mol_plan* plan, int code, const std::string& msg) {
    if (plan) plan->err = msg;
    return code;
}

int cuda_check(mol_plan* plan, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return MOL_OK;
    cudaGetLastError();
    return set_err(plan, e == cudaErrorMemoryAllocation ? MOL_ERR_OOM : MOL_ERR_CUDA,
                   std::string(what) + ": " + cudaGetErrorString(e));
}

bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Device-accessible address of pinned (page-locked, registered or cudaHostAlloc'd) host
// memory, or nullptr for anything else.  On GB300 the GPU reads and writes such memory
// coherently over NVLink-C2C.
void* mapped_host_ptr(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int plan_alloc(mol_plan* plan, void** ptr, size_t bytes) {
    *ptr = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(ptr, bytes);
    if (e != cudaSuccess) return cuda_check(plan, e, "cudaMalloc");
    plan->allocs.push_back(*ptr);
    return MOL_OK;
}

int plan_grid(const mol_plan* plan) { return plan->nblocks; }

// Grid of a grid-stride kernel: a multiple of the SM count when the problem fills
// the machine, otherwise one block per kThreads cells.
int grid_for(long long ncell, int sms, int blocks_per_sm) {
    const long long full = (long long)sms * blocks_per_sm;
    const long long want = (ncell + kThreads - 1) / kThreads;
    return (int)std::max<long long>(1, std::min<long long>(want, full));
}

// Threads per block: kThreads, or fewer for problems smaller than one full wave so that
// every SM gets about the same number of cells (a multiple of 32, at least 64).  Below one
// wave the busiest SM sets the time of an FP64-bound stage, and it issues every warp it holds
// whatever the warp's active lanes: among b = blocks_per_sm .. 1 CTAs per SM the shape whose
// busiest SM holds the fewest warps is taken (65,536 cells on 152 SMs: 293 CTAs of 224 threads,
// 14 warps on the busiest SM, instead of 410 of 160, 15 warps).
int threads_for(long long ncell, int sms, int blocks_per_sm) {
    const long long slots = (long long)sms * blocks_per_sm;
    if (ncell >= slots * kThreads) return kThreads;
    long long best_t = 0, best_w = 0;
    for (int b = blocks_per_sm; b >= 1; --b) {
        const long long sl = (long long)sms * b;
        long long t = (ncell + sl - 1) / sl;
        t = std::max<long long>(64, std::min<long long>(kThreads, (t + 31) / 32 * 32));
        const long long blocks = (ncell + t - 1) / t;
        const long long w = (blocks + sms - 1) / sms * (t / 32);
        if (!best_t || w < best_w) {
            best_t = t;
            best_w = w;
        }
    }
    return (int)best_t;
}

template <class T>
int ensure_ws(mol_plan* plan, int count) {
    T** ws = workspace<T>(plan);
    for (int i = 0; i < count; ++i) {
        if (!ws[i]) {
            void* p;
            int st = plan_alloc(plan, &p, sizeof(T) * (size_t)plan->nunk);
            if (st) return st;
            ws[i] = (T*)p;
        }
    }
    return MOL_OK;
}
template int ensure_ws<double>(mol_plan*, int);
template int ensure_ws<float>(mol_plan*, int);

// allocate one workspace slot only (host staging buffers)
template <class T>
static int ensure_slot(mol_plan* plan, int slot) {
    T** ws = workspace<T>(plan);
    if (ws[slot]) return MOL_OK;
    void* p;
    int st = plan_alloc(plan, &p, sizeof(T) * (size_t)plan->nunk);
    if (st) return st;
    ws[slot] = (T*)p;
    return MOL_OK;
}

// ----------------------------------------------------------------------------
// kernels that do not evaluate the right-hand side (the others are in mol_kernels.cuh)
// ----------------------------------------------------------------------------

// After the controller: commit an accepted step (u <- y7, k1 <- k7), rescale the
// tableau for the new dt and form y2 = u + dt a21 k1 for the next attempt.
template <class T>
__global__ void __launch_bounds__(kThreads) k_tsit_commit(const __grid_constant__ DevProb<T> P, T* u, T* k1, const T* k7, const T* y7,
                                                          T* y2, SolverState* S, int first) {
    const bool acc = !first && S->accepted;
    const bool done = S->done;
    __shared__ double a21;
    if (threadIdx.x == 0) {
        double dt = S->dt;
        a21 = dt * 0.161;
    }
    __syncthreads();
    const long long n = P.ncell * P.nfields;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        T uu, kk;
        if (acc) {
            uu = y7[g];
            kk = k7[g];
            u[g] = uu;
            k1[g] = kk;
        } else {
            uu = u[g];
            kk = k1[g];
        }
        if (!done) y2[g] = fma(T(a21), kk, uu);
    }
    // the tableau is rescaled by the last block once everyone has read S->dt
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned v = atomicAdd(&S->blocks_done, 1u);
        if (v == gridDim.x - 1) {
            tsit_scale(S);
            S->blocks_done = 0;
            __threadfence();
        }
    }
}

// Sums for Hairer's initial step: sums[0] = sum (u/sk)^2, sums[1] = sum (f/sk)^2,
// sums[2] = sum ((f1-f0)/sk)^2 with sk = abstol + |u0| reltol.
template <class T>
__global__ void k_init_norms(long long n, const T* u0, const T* f0, const T* f1, double abstol, double reltol,
                             double* partials) {
    double s0 = 0, s1 = 0, s2 = 0;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        const double sk = abstol + fabs((double)u0[g]) * reltol;
        const double a = (double)u0[g] / sk, b = (double)f0[g] / sk;
        s0 += a * a;
        s1 += b * b;
        if (f1) {
            const double c = ((double)f1[g] - (double)f0[g]) / sk;
            s2 += c * c;
        }
    }
    __shared__ double red[3][kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_down_sync(0xffffffffu, s0, o);
        s1 += __shfl_down_sync(0xffffffffu, s1, o);
        s2 += __shfl_down_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = s0;
        red[1][threadIdx.x >> 5] = s1;
        red[2][threadIdx.x >> 5] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0, c = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) { a += red[0][w]; b += red[1][w]; c += red[2][w]; }
        partials[3 * blockIdx.x + 0] = a;
        partials[3 * blockIdx.x + 1] = b;
        partials[3 * blockIdx.x + 2] = c;
    }
}

template <class T>
__global__ void k_axpy(long long n, T* y, const T* x, const T* f, double h) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x)
        y[g] = fma(T(h), f[g], x[g]);
}

__global__ void k_tsit_init_state(SolverState* S, double t0, double t1, double dt, double abstol, double reltol,
                                  long long maxiters) {
    S->t = t0;
    S->t1 = t1;
    S->dt = dt;
    S->abstol = abstol;
    S->reltol = reltol;
    S->qold = 1e-4;
    S->EEst = 0;
    S->dtmin = 1e-14 * fmax(fabs(t0), fabs(t1)) + 1e-300;
    S->naccept = S->nreject = 0;
    S->nf = 0;
    S->iter = 0;
    S->maxiters = maxiters;
    S->done = (t0 >= t1);
    S->status = 0;
    S->accepted = 0;
    S->blocks_done = 0;
    tsit_scale(S);
}

__global__ void k_set_time(SolverState* S, double t) {
    S->t = t;
    S->blocks_done = 0;
    S->done = 0;
    S->status = 0;
}

// ----------------------------------------------------------------------------
// launch helpers
// ----------------------------------------------------------------------------

// Face buffer of the face pass (allocated on first use, before any graph capture).
template <class T>
T*& face_buf(mol_plan* plan);
template <>
double*& face_buf<double>(mol_plan* plan) { return plan->faces64; }
template <>
float*& face_buf<float>(mol_plan* plan) { return plan->faces32; }

// The face pass runs for FP64 state with generated code only.
template <class T>
bool face_pass_on(const mol_plan* plan) {
    return std::is_same<T, double>::value && plan->face_pass && plan->use_jit;
}

template <class T>
int ensure_faces(mol_plan* plan) {
    if (!std::is_same<T, double>::value || !plan->face_pass || face_buf<T>(plan)) return MOL_OK;
    void* q = nullptr;
    int st = plan_alloc(plan, &q, sizeof(T) * (size_t)plan->nface * (size_t)plan->ncell);
    if (!st) face_buf<T>(plan) = (T*)q;
    return st;
}

// The face pass on state u at S->t + toff (tfix NaN) or tfix + toff; returns the problem
// view the following cell kernel takes (faces set), or the plain view without a face pass.
template <class T>
DevProb<T> with_faces(mol_plan* plan, const T* u, const T* p, double toff, double tfix, cudaError_t* e) {
    DevProb<T> P = prob<T>(plan);
    *e = cudaSuccess;
    T* fb = face_buf<T>(plan);
    cudaKernel_t k = std::is_same<T, double>::value ? plan->jit.faces64 : plan->jit.faces32;
    // FP32 arithmetic is not the bound of the Float32-state kernels: no face pass there
    if (!std::is_same<T, double>::value || !plan->face_pass || !plan->use_jit || !fb || !k) return P;
    *e = launch_k(k, plan->face_blocks > 0 ? plan->face_blocks : plan->nblocks,
                  plan->face_blocks > 0 ? plan->face_threads : plan->nthreads, plan->stream, P, u, p,
                  (const SolverState*)plan->d_state, toff,
                  tfix, fb);
    ++g_launches;
    P.faces = fb;
    return P;
}

template int ensure_faces<double>(mol_plan*);
template int ensure_faces<float>(mol_plan*);
template DevProb<double> with_faces<double>(mol_plan*, const double*, const double*, double, double, cudaError_t*);
template DevProb<float> with_faces<float>(mol_plan*, const float*, const float*, double, double, cudaError_t*);

// The generated forward group of precision T, loaded on first use.  The FP32 group is compiled
// for more resident CTAs per SM than the FP64 one, so its grid is shaped from its own register
// count the first time it is loaded.
template <class T>
int ensure_fwd(mol_plan* plan) {
    const bool is64 = std::is_same<T, double>::value;
    int st = jit_ensure(&plan->jit, is64 ? JIT_FWD64 : JIT_FWD32, plan->jit_err);
    if (st) return set_err(plan, st, plan->jit_err);
    if (!is64 && plan->nblocks32 == 0) {
        plan->nblocks32 = plan->nblocks;
        plan->nthreads32 = plan->nthreads;
        cudaFuncAttributes fa;
        if (cudaFuncGetAttributes(&fa, (const void*)plan->jit.ssp32[0]) == cudaSuccess && fa.numRegs > 0) {
            const int bps = std::max(1, std::min(8, 65536 / (fa.numRegs * kThreads)));
            plan->nthreads32 = threads_for(plan->ncell, plan->sms, bps);
            const long long slots = (long long)plan->sms * bps;
            plan->nblocks32 = (int)std::max<long long>(
                1, std::min<long long>(slots, (plan->ncell + plan->nthreads32 - 1) / plan->nthreads32));
        } else {
            cudaGetLastError();
        }
    }
    return MOL_OK;
}

// Grid of the generated kernels of precision T.
template <class T>
int blocks_of(const mol_plan* plan) {
    return (!std::is_same<T, double>::value && plan->nblocks32 > 0) ? plan->nblocks32 : plan->nblocks;
}
template <class T>
int threads_of(const mol_plan* plan) {
    return (!std::is_same<T, double>::value && plan->nthreads32 > 0) ? plan->nthreads32 : plan->nthreads;
}

template <class T>
int launch_rhs(mol_plan* plan, T* du, const T* u, const T* p, double t) {
    const bool is64 = std::is_same<T, double>::value;
    if (plan->use_jit) {
        int st = ensure_fwd<T>(plan);
        if (st) return st;
        cudaError_t e;
        const DevProb<T> Pf = with_faces<T>(plan, u, p, 0.0, t, &e);
        if (e != cudaSuccess) return cuda_check(plan, e, "face pass launch");
        ++g_launches;
        return cuda_check(plan, launch_k(is64 ? plan->jit.rhs64 : plan->jit.rhs32, blocks_of<T>(plan),
                                         threads_of<T>(plan), plan->stream, Pf, u, du, p, t), "rhs launch");
    }
    k_rhs_t<T, InterpCell><<<plan->nblocks, kThreads, 0, plan->stream>>>(prob<T>(plan), u, du, p, t);
    ++g_launches;
    return cuda_check(plan, cudaGetLastError(), "k_rhs launch");
}
template int launch_rhs<double>(mol_plan*, double*, const double*, const double*, double);
template int launch_rhs<float>(mol_plan*, float*, const float*, const float*, double);

template <class T>
int launch_ssprk_step(mol_plan* plan, T* u, T* u1, T* u2, const T* p, double dt) {
    return launch_ssprk_step_io<T>(plan, u, u, u1, u2, p, dt);
}
template int launch_ssprk_step<double>(mol_plan*, double*, double*, double*, const double*, double);
template int launch_ssprk_step<float>(mol_plan*, float*, float*, float*, const float*, double);

// One SSPRK33 step from uin to uout (which may be the same array).
template <class T>
int launch_ssprk_step_io(mol_plan* plan, const T* uin, T* uout, T* u1, T* u2, const T* p, double dt, bool skip1) {
    const DevProb<T>& P = prob<T>(plan);
    const T* u = uin;
    g_launches += 3;
    if (plan->use_jit) {
        const bool is64 = std::is_same<T, double>::value;
        int st = ensure_fwd<T>(plan);
        if (st) return st;
        const int nb = blocks_of<T>(plan), nt = threads_of<T>(plan);
        cudaKernel_t* k = is64 ? plan->jit.ssp64 : plan->jit.ssp32;
        const T* cu = u;
        const T* cu1 = u1;
        const T* cu2 = u2;
        const double nan = std::nan("");
        cudaError_t e;
        DevProb<T> Pf = with_faces<T>(plan, cu, p, 0.0, nan, &e);
        const long long c0 = 0, c1 = plan->ncell;
        if (e == cudaSuccess && !skip1)
            e = launch_k(k[0], nb, nt, plan->stream, Pf, cu, cu, u1, p, plan->d_state, dt, nan,
                         c0, c1);
        if (e == cudaSuccess) Pf = with_faces<T>(plan, cu1, p, dt, nan, &e);
        if (e == cudaSuccess)
            e = launch_k(k[1], nb, nt, plan->stream, Pf, cu1, cu, u2, p, plan->d_state, dt, nan,
                         c0, c1);
        if (e == cudaSuccess) Pf = with_faces<T>(plan, cu2, p, dt / 2, nan, &e);
        if (e == cudaSuccess)
            e = launch_k(k[2], nb, nt, plan->stream, Pf, cu2, cu, uout, p, plan->d_state, 2 * dt, nan,
                         c0, c1);
        return cuda_check(plan, e, "ssprk launch");
    }
    const double nan = std::nan("");
    const long long c1 = plan->ncell;
    if (!skip1)
        k_ssprk_t<T, InterpCell, 1><<<plan->nblocks, kThreads, 0, plan->stream>>>(P, u, u, u1, p, plan->d_state, dt, nan,
                                                                                   0ll, c1);
    k_ssprk_t<T, InterpCell, 2><<<plan->nblocks, kThreads, 0, plan->stream>>>(P, u1, u, u2, p, plan->d_state, dt, nan,
                                                                               0ll, c1);
    k_ssprk_t<T, InterpCell, 3><<<plan->nblocks, kThreads, 0, plan->stream>>>(P, u2, u, uout, p, plan->d_state, 2 * dt,
                                                                               nan, 0ll, c1);
    return cuda_check(plan, cudaGetLastError(), "k_ssprk launch");
}

// Stage 1 of a step whose state is arriving from pinned host memory: the copy runs on a
// side stream in slabs of whole slices of the slowest interior dimension, and stage 1 of
// each slab starts as soon as the slabs its stencils reach (`halo` slices either side,
// wrapped along a periodic dimension) have landed, so the host-to-device copy hides under
// stage 1 instead of preceding it.  The arithmetic per cell is the unchunked launch's.
template <class T>
int launch_stage1_streamed(mol_plan* plan, const T* host, T* ud, T* u1, const T* p, double dt, int K) {
    const int D = plan->desc.ndim - 1;
    const long long nsl = plan->desc.npts[D] - plan->desc.lower[D] - plan->desc.upper[D];
    const long long S = plan->ncell / nsl;  // cells per slice
    const long long h = plan->halo;
    const bool per = plan->per_last;
    int st;
    if (!plan->copy_stream) {
        if ((st = cuda_check(plan, cudaStreamCreateWithFlags(&plan->copy_stream, cudaStreamNonBlocking), "copy stream")))
            return st;
        for (int k = 0; k <= kMaxSlabs; ++k)
            if ((st = cuda_check(plan, cudaEventCreateWithFlags(&plan->slab_ev[k], cudaEventDisableTiming), "slab event")))
                return st;
    }
    // the copies may only overwrite the staging buffer once earlier work on the stream is done
    if ((st = cuda_check(plan, cudaEventRecord(plan->slab_ev[kMaxSlabs], plan->stream), "record"))) return st;
    if ((st = cuda_check(plan, cudaStreamWaitEvent(plan->copy_stream, plan->slab_ev[kMaxSlabs], 0), "wait"))) return st;
    // slices [s0, s1) of every field in one strided copy (fields are ncell apart)
    auto copy = [&](long long s0, long long s1) -> int {
        if (s1 <= s0) return MOL_OK;
        const size_t pitch = sizeof(T) * (size_t)plan->ncell;
        cudaError_t e = cudaMemcpy2DAsync(ud + s0 * S, pitch, host + s0 * S, pitch, sizeof(T) * (size_t)((s1 - s0) * S),
                                          (size_t)plan->nfields, cudaMemcpyHostToDevice, plan->copy_stream);
        return e == cudaSuccess ? MOL_OK : cuda_check(plan, e, "H2D slab");
    };
    const DevProb<T>& P = prob<T>(plan);
    const double nan = std::nan("");
    const bool is64 = std::is_same<T, double>::value;
    auto stage1 = [&](long long c0, long long c1) -> int {
        if (c1 <= c0) return MOL_OK;
        const int thr = plan->use_jit ? threads_of<T>(plan) : kThreads;
        const int blocks = (int)std::min<long long>(blocks_of<T>(plan), (c1 - c0 + thr - 1) / thr);
        ++g_launches;
        if (plan->use_jit) {
            cudaKernel_t kk = is64 ? plan->jit.ssp64[0] : plan->jit.ssp32[0];
            return cuda_check(plan, launch_k(kk, blocks, thr, plan->stream, P, (const T*)ud, (const T*)ud, u1,
                                             p, plan->d_state, dt, nan, c0, c1), "stage-1 slab");
        }
        k_ssprk_t<T, InterpCell, 1><<<blocks, kThreads, 0, plan->stream>>>(P, ud, ud, u1, p, plan->d_state, dt, nan,
                                                                            c0, c1);
        return cuda_check(plan, cudaGetLastError(), "stage-1 slab");
    };
    // Slab boundaries b[k]; along a periodic dimension the last `halo` slices travel first,
    // since the first slices read them through the wrap.  Stage 1 of the window
    // [b[k] - halo, b[k+1] - halo) reads slices below b[k+1] only, so it runs as soon as slab k
    // has landed (the last window runs to the end): each launch is issued right behind its
    // copy, and only the last window waits for the whole state.
    std::vector<long long> b(K + 1);
    for (int k = 0; k <= K; ++k) b[k] = nsl * k / K;
    const long long tail = per ? std::min(h, nsl) : 0;
    if ((st = copy(nsl - tail, nsl))) return st;
    for (int k = 0; k < K; ++k) {
        const long long s1 = std::min(b[k + 1], nsl - tail);
        if ((st = copy(std::min(b[k], s1), s1))) return st;
        if ((st = cuda_check(plan, cudaEventRecord(plan->slab_ev[k], plan->copy_stream), "record"))) return st;
        if ((st = cuda_check(plan, cudaStreamWaitEvent(plan->stream, plan->slab_ev[k], 0), "wait slab"))) return st;
        const long long w0 = std::max(0ll, b[k] - h), w1 = k == K - 1 ? nsl : std::max(0ll, b[k + 1] - h);
        if ((st = stage1(w0 * S, w1 * S))) return st;
    }
    // the remaining stages read the whole state: every slab is in once the last event is
    return cuda_check(plan, cudaStreamWaitEvent(plan->stream, plan->slab_ev[K - 1], 0), "wait last slab");
}
template int launch_ssprk_step_io<double>(mol_plan*, const double*, double*, double*, double*, const double*, double,
                                          bool);
template int launch_ssprk_step_io<float>(mol_plan*, const float*, float*, float*, float*, const float*, double, bool);

// Every point of the full grid: unknowns, observed boundary values (boundary rows, extrapolated
// points, ghost points of edge-aligned grids), periodic images and corner points (0), field-major
// with the first dimension fastest: the arrays behind sol[u(t, x)] of the reference's
// PDETimeSeriesSolution (interface/solution/timedep.jl:19-80), resolved exactly as the
// right-hand side's taps are (load_pt).
template <class T>
__global__ void __launch_bounds__(kThreads) k_fill_grid_t(const __grid_constant__ DevProb<T> P,
                                                          const T* __restrict__ u, const T* __restrict__ p, T t,
                                                          T* __restrict__ full, long long per_field) {
    const long long total = per_field * P.nfields;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < total;
         g += (long long)gridDim.x * blockDim.x) {
        const int f = (int)(g / per_field);
        long long r = g - (long long)f * per_field;
        const int i0 = (int)(r % P.n[0]);
        r /= P.n[0];
        const int i1 = (int)(r % P.n[1]);
        const int i2 = (int)(r / P.n[1]);
        // outside the interior box in two or more dimensions, periodic images included, is a
        // corner (~ 0): the periodic and boundary rows cover only the interior's edge slices
        // (generate_bc_eqs.jl:35-58, :396-459)
        const int I[3] = {i0 + 1, i1 + 1, i2 + 1};
        int nout = 0;
#pragma unroll
        for (int d = 0; d < 3; ++d) nout += (I[d] <= P.lo[d]) | (I[d] > P.n[d] - P.up[d]);
        full[g] = nout > 1 ? T(0) : load_pt(P, u, f, I[0], I[1], I[2], t, p);
    }
}


}  // namespace mol

using namespace mol;

// ----------------------------------------------------------------------------
// descriptor validation
// ----------------------------------------------------------------------------

static int validate_prog(mol_plan* plan, const mol_problem_desc* d, int prog, int kind, int nregs,
                         long long aux_need_cell, const mol_term* term) {
    if (prog < 0 || prog >= d->nprogs) return set_err(plan, MOL_ERR_INVALID, "program index out of range");
    const int start = d->prog_ranges[2 * prog], len = d->prog_ranges[2 * prog + 1];
    if (start < 0 || len < 0 || start + len > d->ninstr) return set_err(plan, MOL_ERR_INVALID, "program range out of bounds");
    for (int pc = start; pc < start + len; ++pc) {
        const mol_instr& in = d->code[pc];
        const bool bc_are_terms = in.op == MOL_OP_UPWIND;
        if (in.dst >= nregs || in.a >= nregs || (!bc_are_terms && (in.b >= nregs || in.c >= nregs)))
            return set_err(plan, MOL_ERR_INVALID, "register index out of range");
        switch (in.op) {
            case MOL_OP_CONST:
                if (in.imm < 0 || in.imm >= d->nconsts) return set_err(plan, MOL_ERR_INVALID, "constant index");
                break;
            case MOL_OP_PARAM:
                if (in.imm < 0 || in.imm >= d->nparams) return set_err(plan, MOL_ERR_INVALID, "parameter index");
                break;
            case MOL_OP_FIELD:
                if (kind == 2) return set_err(plan, MOL_ERR_INVALID, "FIELD in a boundary program");
                if (in.imm < 0 || in.imm >= d->nfields) return set_err(plan, MOL_ERR_INVALID, "field index");
                break;
            case MOL_OP_AUX: {
                const int ax = kind == 1 ? term->aux0 + in.imm : in.imm;
                if (ax < 0 || ax >= d->naux) return set_err(plan, MOL_ERR_INVALID, "aux index");
                long long need = aux_need_cell;
                if (kind == 2) {  // boundary programs read full-grid arrays at the boundary point
                    need = 1;
                    for (int q = 0; q < d->ndim; ++q) need *= d->npts[q];
                } else if (kind == 1) {
                    need = 1;
                    for (int q = 0; q < 3; ++q)
                        need *= (q < d->ndim ? d->npts[q] : 1) + (q == term->dim ? 1 : 0);
                }
                if (d->aux_len[ax] < need) return set_err(plan, MOL_ERR_INVALID, "aux array too short");
                break;
            }
            case MOL_OP_COORD:
                if (kind == 1) return set_err(plan, MOL_ERR_INVALID, "COORD in a face program (hoist it)");
                if (in.imm < 0 || in.imm >= d->ndim) return set_err(plan, MOL_ERR_INVALID, "coordinate index");
                break;
            case MOL_OP_TIME: break;
            case MOL_OP_TERM:
                if (kind != 0 || in.imm < 0 || in.imm >= d->nterms) return set_err(plan, MOL_ERR_INVALID, "term index");
                break;
            case MOL_OP_UPWIND:
                if (kind != 0 || in.b >= d->nterms || in.c >= d->nterms) return set_err(plan, MOL_ERR_INVALID, "upwind terms");
                break;
            case MOL_OP_ADD: case MOL_OP_SUB: case MOL_OP_MUL: case MOL_OP_DIV: case MOL_OP_NEG:
            case MOL_OP_POWI: case MOL_OP_POW: case MOL_OP_IFELSE:
                break;
            case MOL_OP_FN:
                if (in.imm < 0 || in.imm > MOL_FN_ATAN) return set_err(plan, MOL_ERR_INVALID, "function id");
                break;
            case MOL_OP_CMP:
                if (in.imm < 0 || in.imm > MOL_CMP_EQ) return set_err(plan, MOL_ERR_INVALID, "comparison id");
                break;
            case MOL_OP_OUT:
                if (kind == 0 && (in.imm < 0 || in.imm >= d->nfields)) return set_err(plan, MOL_ERR_INVALID, "output index");
                if (kind == 2 && (in.imm < 0 || in.imm > 2)) return set_err(plan, MOL_ERR_INVALID, "output index");
                break;
            default:
                return set_err(plan, MOL_ERR_INVALID, "unknown opcode");
        }
    }
    return MOL_OK;
}

static int validate_desc(mol_plan* plan, const mol_problem_desc* d) {
    if (!d) return set_err(plan, MOL_ERR_INVALID, "null descriptor");
    if (d->abi_version != MOL_ABI_VERSION) return set_err(plan, MOL_ERR_INVALID, "ABI version mismatch");
    if (d->ndim < 1 || d->ndim > MOL_MAX_DIMS) return set_err(plan, MOL_ERR_INVALID, "ndim must be 1..3");
    if (d->nfields < 1 || d->nfields > MOL_MAX_FIELDS) return set_err(plan, MOL_ERR_INVALID, "nfields must be 1..8");
    if (d->nparams < 0 || (d->nparams > 0 && !d->params)) return set_err(plan, MOL_ERR_INVALID, "parameters");
    for (int q = 0; q < d->ndim; ++q) {
        if (d->npts[q] < 1 || d->npts[q] > (1ll << 30)) return set_err(plan, MOL_ERR_INVALID, "npts out of range");
        if (d->lower[q] < 0 || d->upper[q] < 0 || d->npts[q] - d->lower[q] - d->upper[q] < 1)
            return set_err(plan, MOL_ERR_INVALID, "empty interior");
        if (!d->coords[q]) return set_err(plan, MOL_ERR_INVALID, "missing coordinates");
    }
    if (d->nops < 0 || (d->nops && !d->ops)) return set_err(plan, MOL_ERR_INVALID, "ops");
    for (int i = 0; i < d->nops; ++i) {
        const mol_op1d& o = d->ops[i];
        if (o.L < 0 || o.nlo < 0 || o.nhi < 0 || o.bLlo < 0 || o.bLhi < 0 || o.hi_base < 0 || o.hi_base > 1 ||
            o.nrows < 0)
            return set_err(plan, MOL_ERR_INVALID, "operator sizes");
        if (o.w_int < 0 || o.w_int + (long long)std::max(1, o.nrows) * o.L > d->nweights || o.w_lo < 0 ||
            o.w_lo + (long long)o.nlo * o.bLlo > d->nweights || o.w_hi < 0 ||
            o.w_hi + (long long)o.nhi * o.bLhi > d->nweights)
            return set_err(plan, MOL_ERR_INVALID, "operator weights out of the pool");
    }
    if (d->nterms < 0 || (d->nterms && !d->terms)) return set_err(plan, MOL_ERR_INVALID, "terms");
    for (int k = 0; k < d->nterms; ++k) {
        const mol_term& t = d->terms[k];
        if (t.field < 0 || t.field >= d->nfields || t.dim < 0 || t.dim >= d->ndim)
            return set_err(plan, MOL_ERR_INVALID, "term field/dim");
        auto opok = [&](int o) { return o >= 0 && o < d->nops; };
        auto rows = [&](int o) { return opok(o) && d->ops[o].nrows > 0; };
        switch (t.kind) {
            case MOL_TERM_LINEAR:
                if (!opok(t.op)) return set_err(plan, MOL_ERR_INVALID, "term op");
                if (rows(t.op)) {
                    const mol_op1d& o = d->ops[t.op];
                    if (d->bc[t.field][t.dim][0].kind == MOL_BC_PERIODIC)
                        return set_err(plan, MOL_ERR_UNSUPPORTED, "per-point operator rows on a periodic dimension");
                    // every interior point that reads an interior row has one: rows up to
                    // position min(n - upper, n - nhi) (row index = position - nlo - 1)
                    const long long n = d->npts[t.dim];
                    if (o.nrows < std::min<long long>(n - d->upper[t.dim], n - o.nhi) - o.nlo)
                        return set_err(plan, MOL_ERR_INVALID, "operator rows do not match the grid");
                }
                break;
            case MOL_TERM_MIXED:
                if (!opok(t.op) || !opok(t.op2) || t.dim2 < 0 || t.dim2 >= d->ndim || t.dim2 == t.dim)
                    return set_err(plan, MOL_ERR_INVALID, "mixed term");
                // nonuniform dimensions (centered_difference.jl:32-56 on each): no wrap, and rows
                // for every interior point that reads an interior row
                for (int q = 0; q < 2; ++q) {
                    const int o = q == 0 ? t.op : t.op2, dm = q == 0 ? t.dim : t.dim2;
                    if (!rows(o)) continue;
                    if (d->bc[t.field][dm][0].kind == MOL_BC_PERIODIC)
                        return set_err(plan, MOL_ERR_UNSUPPORTED, "per-point operator rows on a periodic dimension");
                    const long long n = d->npts[dm];
                    if (d->ops[o].nrows < std::min<long long>(n - d->upper[dm], n - d->ops[o].nhi) - d->ops[o].nlo)
                        return set_err(plan, MOL_ERR_INVALID, "operator rows do not match the grid");
                }
                break;
            case MOL_TERM_WENO:
                if (!(t.dx > 0)) return set_err(plan, MOL_ERR_INVALID, "weno dx");
                if (t.variant == 1) {  // nonuniform: geometry rows for every point, no wrap
                    if (!opok(t.op) || d->ops[t.op].L != 56 || d->ops[t.op].nrows != d->npts[t.dim] ||
                        d->npts[t.dim] < 5)
                        return set_err(plan, MOL_ERR_INVALID, "nonuniform WENO geometry rows");
                    if (d->bc[t.field][t.dim][0].kind == MOL_BC_PERIODIC)
                        return set_err(plan, MOL_ERR_UNSUPPORTED, "nonuniform WENO on a periodic dimension");
                    break;
                }
                if (t.variant != 0) return set_err(plan, MOL_ERR_INVALID, "weno variant");
                // bounded dimension: the interior stops two points from each end and the points
                // next to the boundary points are extrapolated (WENO.jl:94, generate_bc_eqs.jl:336-392);
                // with no boundary row at an end the reference uses its near-wall WENO stencils
                if (d->bc[t.field][t.dim][0].kind != MOL_BC_PERIODIC &&
                    !(d->bc[t.field][t.dim][0].extrap > 0 && d->bc[t.field][t.dim][1].extrap > 0))
                    return set_err(plan, MOL_ERR_UNSUPPORTED,
                                   "WENO on a bounded dimension needs extrapolation rows at both ends "
                                   "(the near-wall nonuniform WENO stencils are not built)");
                if (d->npts[t.dim] - 1 < 5) return set_err(plan, MOL_ERR_INVALID, "WENO needs at least 6 grid points to wrap");
                break;
            case MOL_TERM_NONLINLAP:
                if (!opok(t.op) || !opok(t.op2) || !opok(t.op3)) return set_err(plan, MOL_ERR_INVALID, "nonlinlap ops");
                if (rows(t.op) || rows(t.op2) || rows(t.op3)) {
                    // nonuniform grid (half_offset_centred_difference.jl:39-69): no wrap, and rows
                    // for every position that reads an interior row: the outer operator at
                    // II - 1 on the n - 1 half points, the inner ones at half points up to n - 1
                    if (d->bc[t.field][t.dim][0].kind == MOL_BC_PERIODIC)
                        return set_err(plan, MOL_ERR_UNSUPPORTED, "per-point operator rows on a periodic dimension");
                    const long long n = d->npts[t.dim];
                    const mol_op1d& oo = d->ops[t.op];
                    const mol_op1d& oi = d->ops[t.op2];
                    const mol_op1d& oq = d->ops[t.op3];
                    if ((oo.nrows > 0 && oo.nrows < std::min<long long>(n - 1 - d->upper[t.dim], n - 1 - oo.nhi) - oo.nlo) ||
                        (oi.nrows > 0 && oi.nrows < std::min<long long>(n - 1, n - oi.nhi) - oi.nlo) ||
                        (oq.nrows > 0 && oq.nrows < std::min<long long>(n - 1, n - oq.nhi) - oq.nlo))
                        return set_err(plan, MOL_ERR_INVALID, "operator rows do not match the grid");
                }
                if (t.prog >= 0) {
                    int st = validate_prog(plan, d, t.prog, 1, MOL_MAX_REGS, 0, &t);
                    if (st) return st;
                }
                break;
            default: return set_err(plan, MOL_ERR_INVALID, "unknown term kind");
        }
    }
    if (!d->code || !d->prog_ranges) return set_err(plan, MOL_ERR_INVALID, "programs");
    long long ncell = 1;
    for (int q = 0; q < d->ndim; ++q) ncell *= d->npts[q] - d->lower[q] - d->upper[q];
    int st = validate_prog(plan, d, d->cell_prog, 0, MOL_MAX_REGS, ncell, nullptr);
    if (st) return st;
    for (int f = 0; f < d->nfields; ++f)
        for (int q = 0; q < d->ndim; ++q) {
            const bool per = d->bc[f][q][0].kind == MOL_BC_PERIODIC;
            if (per && d->lower[q] != 1) return set_err(plan, MOL_ERR_INVALID, "periodic dims clip exactly the low point");
            for (int s = 0; s < 2; ++s) {
                const mol_bc& b = d->bc[f][q][s];
                const int clip = s == 0 ? d->lower[q] : d->upper[q];
                if (b.extrap < 0 || b.extrap > d->nops) return set_err(plan, MOL_ERR_INVALID, "extrapolation operator");
                if (b.extrap > 0) {
                    const mol_op1d& x = d->ops[b.extrap - 1];
                    const int rows = s == 0 ? x.nlo : x.nhi, len = s == 0 ? x.bLlo : x.bLhi;
                    if (rows < 2 || len < 3 || len > d->npts[q])
                        return set_err(plan, MOL_ERR_INVALID, "extrapolation table lacks a second row");
                    if (clip != 2 || per)
                        return set_err(plan, MOL_ERR_INVALID, "an extrapolated point needs the interior two points from the end");
                    if (b.kind != MOL_BC_ROBIN)
                        return set_err(plan, MOL_ERR_UNSUPPORTED, "an extrapolated point needs a boundary row at the end point");
                    if (b.prog < 0 && b.b != 0.0)
                        return set_err(plan, MOL_ERR_UNSUPPORTED,
                                       "an extrapolated point next to a Neumann/Robin row (a coupled pair of rows) is not built");
                } else if (clip > 1 && !per) {
                    return set_err(plan, MOL_ERR_UNSUPPORTED, "interior stops more than one point from the end without an extrapolation row");
                }
                if (b.kind == MOL_BC_ROBIN) {
                    if (b.op < 0 || b.op >= d->nops) return set_err(plan, MOL_ERR_INVALID, "bc operator");
                    const mol_op1d& o = d->ops[b.op];
                    if ((s == 0 && (o.nlo < 1 || o.bLlo < 1)) || (s == 1 && (o.nhi < 1 || o.bLhi < 1)))
                        return set_err(plan, MOL_ERR_INVALID, "bc operator lacks a boundary table");
                    if (b.prog >= 0) {
                        st = validate_prog(plan, d, b.prog, 2, 16, 0, nullptr);
                        if (st) return st;
                    }
                } else if (b.kind == MOL_BC_EDGE) {
                    if (per || b.extrap) return set_err(plan, MOL_ERR_INVALID, "edge row on a periodic or extrapolated end");
                    const int n = (int)d->npts[q], pos = s == 0 ? 1 : n - 1, ghost = s == 0 ? 1 : n;
                    for (int o : {b.op, b.iop}) {
                        if (o < 0 || o >= d->nops) return set_err(plan, MOL_ERR_INVALID, "edge bc operator");
                        // the tap window the device selects (select_taps at pos on n points) must hold
                        // the ghost point and otherwise unknowns of this line only
                        const mol_op1d& x = d->ops[o];
                        int first, cnt;
                        if (pos <= x.nlo) { first = 1; cnt = x.bLlo; }
                        else if (pos > n - x.nhi) { first = n - x.bLhi + 1; cnt = x.bLhi; }
                        else { first = pos + x.omin; cnt = x.L; }
                        const int last = first + cnt - 1;
                        if (cnt < 1 || ghost < first || ghost > last || first < 1 || last > n ||
                            (s == 0 && last > n - d->upper[q]) || (s == 1 && first <= d->lower[q]))
                            return set_err(plan, MOL_ERR_INVALID, "edge bc stencil leaves the line");
                    }
                    if (b.prog >= 0) {
                        st = validate_prog(plan, d, b.prog, 2, 16, 0, nullptr);
                        if (st) return st;
                    }
                } else if (b.kind != MOL_BC_NONE && b.kind != MOL_BC_PERIODIC) {
                    return set_err(plan, MOL_ERR_INVALID, "bc kind");
                }
            }
        }
    return MOL_OK;
}

template <class T>
static int upload(mol_plan* plan, void** dst, const double* src, long long n) {
    std::vector<T> tmp((size_t)std::max<long long>(n, 1));
    for (long long i = 0; i < n; ++i) tmp[(size_t)i] = (T)src[i];
    int st = plan_alloc(plan, dst, sizeof(T) * tmp.size());
    if (st) return st;
    return cuda_check(plan, cudaMemcpy(*dst, tmp.data(), sizeof(T) * (size_t)n, cudaMemcpyHostToDevice), "upload");
}

template <class T>
static int build_prec(mol_plan* plan, const mol_problem_desc* d, PlanArrays& A, DevProb<T>& P) {
    int st;
    if ((st = upload<T>(plan, &A.w, d->weights, d->nweights))) return st;
    if ((st = upload<T>(plan, &A.consts, d->consts, d->nconsts))) return st;
    std::vector<double> aux((size_t)std::max<long long>(plan->aux_total, 1));
    for (int i = 0; i < d->naux; ++i)
        std::memcpy(aux.data() + plan->aux_off_host[i], d->aux[i], sizeof(double) * (size_t)d->aux_len[i]);
    if ((st = upload<T>(plan, &A.aux, aux.data(), plan->aux_total))) return st;
    for (int q = 0; q < 3; ++q) {
        if (q < d->ndim) {
            if ((st = upload<T>(plan, &A.coords[q], d->coords[q], d->npts[q]))) return st;
        } else {
            double one = 0.0;
            if ((st = upload<T>(plan, &A.coords[q], &one, 1))) return st;
        }
    }
    std::vector<DevBC<T>> bc(MOL_MAX_FIELDS * 3 * 2);
    for (int f = 0; f < MOL_MAX_FIELDS; ++f)
        for (int q = 0; q < 3; ++q)
            for (int s = 0; s < 2; ++s) {
                DevBC<T> b{};
                b.xop = -1;
                if (f < d->nfields && q < d->ndim) {
                    const mol_bc& src = d->bc[f][q][s];
                    b.kind = src.kind;
                    b.prog = src.prog;
                    b.op = src.op;
                    b.xop = src.extrap - 1;
                    b.iop = src.iop;
                    b.a = (T)src.a;
                    b.b = (T)src.b;
                    b.g = (T)src.g;
                    // constant rows: the reciprocal of the solved-for coefficient, and the
                    // Dirichlet value, once on the host (the device multiplies)
                    if (src.kind == MOL_BC_ROBIN && src.prog < 0) {
                        if (b.b == (T)0) {
                            b.c0 = b.g / b.a;
                        } else if (src.op >= 0 && src.op < d->nops) {
                            const mol_op1d& o = d->ops[src.op];
                            const long long wkb = s == 0 ? o.w_lo : o.w_hi + (o.bLhi - 1);
                            const T den = std::fma(b.b, (T)d->weights[wkb], b.a);
                            b.inv = (T)1 / den;
                        }
                    }
                }
                bc[(f * 3 + q) * 2 + s] = b;
            }
    if ((st = plan_alloc(plan, &A.bc, sizeof(DevBC<T>) * bc.size()))) return st;
    if ((st = cuda_check(plan, cudaMemcpy(A.bc, bc.data(), sizeof(DevBC<T>) * bc.size(), cudaMemcpyHostToDevice), "bc")))
        return st;
    if ((st = upload<T>(plan, &A.params, d->params, d->nparams))) return st;
    A.params_host.assign(d->nparams, 0.0);
    for (int i = 0; i < d->nparams; ++i) A.params_host[i] = (double)(T)d->params[i];
    A.params_known = true;
    P.ndim = d->ndim;
    P.nfields = d->nfields;
    P.nparams = d->nparams;
    P.cell_prog = d->cell_prog;
    for (int q = 0; q < 3; ++q) {
        P.n[q] = q < d->ndim ? (int)d->npts[q] : 1;
        P.lo[q] = q < d->ndim ? d->lower[q] : 0;
        P.up[q] = q < d->ndim ? d->upper[q] : 0;
        P.ni[q] = P.n[q] - P.lo[q] - P.up[q];
        P.coords[q] = (const T*)A.coords[q];
    }
    P.fastdiv = plan->ncell < (1ll << 31) && P.ni[0] >= 1 && P.ni[1] >= 1;
    for (int q = 0; q < 2; ++q) divmagic((unsigned)std::max(1, P.ni[q]), &P.dm[q], &P.ds[q]);
    for (int f = 0; f < MOL_MAX_FIELDS; ++f) {
        int m = 0;
        if (f < d->nfields)
            for (int q = 0; q < d->ndim; ++q)
                if (d->bc[f][q][0].kind == MOL_BC_PERIODIC) m |= 1 << q;
        P.permask[f] = m;
    }
    P.ncell = plan->ncell;
    P.faces = nullptr;
    P.cw = nullptr;
    P.fstride = plan->ncell;
    P.fbeg = 0;
    P.fend = plan->ncell;
    P.bc = (const DevBC<T>*)A.bc;
    P.ops = plan->d_ops;
    P.w = (const T*)A.w;
    P.terms = plan->d_terms;
    P.code = plan->d_code;
    P.progs = plan->d_progs;
    P.consts = (const T*)A.consts;
    P.aux = (const T*)A.aux;
    P.aux_off = plan->d_aux_off;
    P.naux = d->naux;
    return MOL_OK;
}

static int copy_struct(mol_plan* plan, void** dst, const void* src, size_t bytes) {
    int st = plan_alloc(plan, dst, bytes);
    if (st) return st;
    if (bytes == 0) return MOL_OK;
    return cuda_check(plan, cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice), "descriptor copy");
}

// ----------------------------------------------------------------------------
// C ABI
// ----------------------------------------------------------------------------

extern "C" {

int mol_version(void) { return MOL_ABI_VERSION * 10000 + 100; }

const char* mol_status_string(int s) {
    switch (s) {
        case MOL_OK: return "ok";
        case MOL_ERR_INVALID: return "invalid descriptor or argument";
        case MOL_ERR_OOM: return "device out of memory";
        case MOL_ERR_NONFINITE: return "non-finite state";
        case MOL_ERR_TIMEOUT: return "device wait timed out";
        case MOL_ERR_CUDA: return "CUDA error";
        case MOL_ERR_UNSUPPORTED: return "unsupported discretization";
        case MOL_ERR_MAXITERS: return "maximum iterations reached";
        case MOL_ERR_DTMIN: return "step size underflow";
        default: return "unknown status";
    }
}

int64_t mol_launch_count(void) { return g_launches.load(); }

int mol_plan_uses_codegen(const mol_plan* plan) { return plan && plan->use_jit ? 1 : 0; }
int mol_plan_coef_arrays(const mol_plan* plan) { return plan ? plan->ncoef : 0; }

int mol_plan_launch_config(const mol_plan* plan, int32_t* regs, int32_t* threads, int32_t* blocks) {
    if (!plan) return MOL_ERR_INVALID;
    int r = 0;
    cudaFuncAttributes fa;
    if (plan->use_jit && plan->jit.ssp64[0] &&
        cudaFuncGetAttributes(&fa, (const void*)plan->jit.ssp64[0]) == cudaSuccess)
        r = fa.numRegs;
    else
        cudaGetLastError();
    if (regs) *regs = r;
    if (threads) *threads = plan->use_jit ? plan->nthreads : kThreads;
    if (blocks) *blocks = plan->nblocks;
    return MOL_OK;
}

const char* mol_plan_codegen_source(const mol_plan* plan) {
    if (!plan) return "";
    return plan->use_jit ? plan->jit_src.c_str() : plan->jit_err.c_str();
}

const char* mol_last_error(const mol_plan* plan) { return plan ? plan->err.c_str() : "null plan"; }

int64_t mol_plan_n_unknowns(const mol_plan* plan) { return plan ? plan->nunk : -1; }

int mol_plan_set_stream(mol_plan* plan, void* stream) {
    if (!plan) return MOL_ERR_INVALID;
    if (plan->own_stream && plan->stream) cudaStreamDestroy(plan->stream);
    plan->own_stream = false;
    plan->stream = (cudaStream_t)stream;
    if (plan->g_ssp64) { cudaGraphExecDestroy(plan->g_ssp64); plan->g_ssp64 = nullptr; }
    if (plan->g_ssp32) { cudaGraphExecDestroy(plan->g_ssp32); plan->g_ssp32 = nullptr; }
    return MOL_OK;
}

int mol_plan_destroy(mol_plan* plan) {
    if (!plan) return MOL_ERR_INVALID;
    cudaSetDevice(plan->dev);
    if (plan->stream) cudaStreamSynchronize(plan->stream);
    if (plan->g_ssp64) cudaGraphExecDestroy(plan->g_ssp64);
    if (plan->g_ssp32) cudaGraphExecDestroy(plan->g_ssp32);
    for (void* p : plan->allocs) cudaFree(p);
    if (plan->copy_stream) {
        cudaStreamSynchronize(plan->copy_stream);
        cudaStreamDestroy(plan->copy_stream);
    }
    for (cudaEvent_t e : plan->slab_ev)
        if (e) cudaEventDestroy(e);
    if (plan->own_stream && plan->stream) cudaStreamDestroy(plan->stream);
    delete plan;
    return MOL_OK;
}

int mol_generate_code(const mol_problem_desc* desc, char* buf, int64_t bufsize, int64_t* needed) {
    mol_plan tmp;
    int st = validate_desc(&tmp, desc);
    if (st) return st;
    std::string why;
    const std::string src = generate_source(desc, why);
    if (src.empty()) return MOL_ERR_UNSUPPORTED;
    if (needed) *needed = (int64_t)src.size() + 1;
    if (buf && bufsize > 0) {
        const size_t n = std::min<size_t>((size_t)bufsize - 1, src.size());
        std::memcpy(buf, src.data(), n);
        buf[n] = 0;
    }
    return MOL_OK;
}

int mol_codegen_compile_check(const mol_problem_desc* desc, char* log, int64_t logsize) {
    mol_plan tmp;
    int st = validate_desc(&tmp, desc);
    std::string err = tmp.err;
    if (!st) {
        std::string why;
        const std::string src = generate_source(desc, why);
        if (src.empty()) {
            st = MOL_ERR_UNSUPPORTED;
            err = why;
        } else {
            for (int grp = 0; grp < 4 && !st; ++grp) st = nvrtc_compile(src, desc->nparams, grp, nullptr, nullptr, err);
        }
    }
    if (log && logsize > 0) {
        const size_t n = std::min<size_t>((size_t)logsize - 1, err.size());
        std::memcpy(log, err.data(), n);
        log[n] = 0;
    }
    return st;
}

int mol_plan_create(const mol_problem_desc* d, mol_plan** out) { return mol::plan_create_impl(d, out, false); }

}  // extern "C"

// `member` plans belong to an ensemble: no stream, no solver workspace, no code
// generation of their own (the ensemble compiles one module for all members).
int mol::plan_create_impl(const mol_problem_desc* d, mol_plan** out, bool member) {
    if (!out) return MOL_ERR_INVALID;
    *out = nullptr;
    mol_plan* plan = new mol_plan();
    int st = validate_desc(plan, d);
    if (st) {
        *out = plan;  // caller may read mol_last_error, then destroy
        return st;
    }
    cudaGetDevice(&plan->dev);
    plan->desc = *d;
    plan->nfields = d->nfields;
    plan->nparams = d->nparams;
    plan->naux = d->naux;
    long long ncell = 1;
    for (int q = 0; q < d->ndim; ++q) ncell *= d->npts[q] - d->lower[q] - d->upper[q];
    plan->ncell = ncell;
    plan->nunk = ncell * d->nfields;
    plan->aux_off_host.resize(d->naux + 1);
    long long off = 0;
    for (int i = 0; i < d->naux; ++i) {
        plan->aux_off_host[i] = off;
        off += d->aux_len[i];
    }
    plan->aux_off_host[d->naux] = off;
    plan->aux_total = off;
    plan->params_host.assign(d->params, d->params + d->nparams);
    auto fail = [&](int code) {
        *out = plan;
        return code;
    };
    // Derived copies the kernels use: product weights of every mixed derivative appended
    // to the pool (term.reserved0 = their offset, row-major [L1][L2]) and 1/dx in WENO terms.
    std::vector<double> weights(d->weights, d->weights + d->nweights);
    std::vector<mol_term> terms(d->terms, d->terms + d->nterms);
    for (int k = 0; k < d->nterms; ++k) {
        mol_term& tm = terms[k];
        if (tm.kind == MOL_TERM_MIXED) {
            const mol_op1d& o1 = d->ops[tm.op];
            const mol_op1d& o2 = d->ops[tm.op2];
            tm.reserved0 = (int32_t)weights.size();
            for (int x = 0; x < o1.L; ++x)
                for (int y = 0; y < o2.L; ++y) weights.push_back(d->weights[o1.w_int + x] * d->weights[o2.w_int + y]);
        } else if (nonlinlap_fold(d, k)) {
            // folded nonlinear Laplacian: the cell's scale wo[1] wi[1] and the face's 1 / wi[1]
            const double wo1 = d->weights[d->ops[tm.op].w_int + 1], wi1 = d->weights[d->ops[tm.op2].w_int + 1];
            tm.reserved0 = (int32_t)weights.size();
            weights.push_back(wo1 * wi1);
            weights.push_back(1.0 / wi1);
        }
    }
    // fused weights of the constant-coefficient first-derivative groups (at reserved2 of
    // each group's key term)
    for (const FoldGroup& g : const_linear_groups(d)) {
        const std::vector<double> fw = fold_weights(d, g);
        terms[g.key_term].reserved2 = (int32_t)weights.size();
        weights.insert(weights.end(), fw.begin(), fw.end());
    }
    mol_problem_desc dd = *d;
    dd.weights = weights.data();
    dd.nweights = (int64_t)weights.size();
    dd.terms = terms.data();
    std::vector<mol_term> dev_terms = terms;
    for (auto& tm : dev_terms)
        if (tm.kind == MOL_TERM_WENO) tm.dx = 1.0 / tm.dx;
    d = &dd;
    if (!member) {
        if ((st = cuda_check(plan, cudaStreamCreateWithFlags(&plan->stream, cudaStreamNonBlocking), "stream")))
            return fail(st);
        plan->own_stream = true;
    }
    if ((st = copy_struct(plan, (void**)&plan->d_ops, d->ops, sizeof(mol_op1d) * d->nops))) return fail(st);
    if ((st = copy_struct(plan, (void**)&plan->d_terms, dev_terms.data(), sizeof(mol_term) * d->nterms)))
        return fail(st);
    if ((st = copy_struct(plan, (void**)&plan->d_code, d->code, sizeof(mol_instr) * d->ninstr))) return fail(st);
    if ((st = copy_struct(plan, (void**)&plan->d_progs, d->prog_ranges, sizeof(int) * 2 * d->nprogs))) return fail(st);
    if ((st = copy_struct(plan, (void**)&plan->d_aux_off, plan->aux_off_host.data(), sizeof(long long) * (d->naux + 1))))
        return fail(st);
    if ((st = build_prec<double>(plan, d, plan->a64, plan->P64))) return fail(st);
    if ((st = build_prec<float>(plan, d, plan->a32, plan->P32))) return fail(st);
    if (member) {
        *out = plan;
        return MOL_OK;
    }
    if ((st = plan_alloc(plan, (void**)&plan->d_state, sizeof(SolverState)))) return fail(st);
    cudaMemset(plan->d_state, 0, sizeof(SolverState));
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, plan->dev);
    plan->sms = sms;
    // provisional grid (refined once the kernels' register use is known)
    plan->nblocks = grid_for(ncell, sms, 2);
    if ((st = plan_alloc(plan, (void**)&plan->d_partials, sizeof(double) * 3 * (size_t)sms * 8))) return fail(st);
    // the generated right-hand side; MOL_DISABLE_CODEGEN=1 keeps the interpreter (used to cross-check)
    const char* off_env = getenv("MOL_DISABLE_CODEGEN");
    if (!(off_env && off_env[0] == '1')) {
        // Resident CTAs per SM the register allocator must allow: 3 for large problems (hides
        // more load latency), 2 below a million unknowns (measured on GB300).
        const int minb = plan->nunk >= (1ll << 20) ? 3 : 2;
        st = jit_compile(d, &plan->jit, plan->jit_err, &plan->jit_src, minb);
        plan->use_jit = (st == MOL_OK) && plan->jit.ok;
        if (plan->use_jit) {
            // Grid = SMs x resident CTAs: every SM gets the same share of the grid-stride loop.
            cudaFuncAttributes fa;
            if (cudaFuncGetAttributes(&fa, (const void*)plan->jit.ssp64[0]) == cudaSuccess && fa.numRegs > 0) {
                const int bps = std::max(1, std::min(8, 65536 / (fa.numRegs * kThreads)));
                plan->nthreads = threads_for(ncell, sms, bps);
                const long long slots = (long long)sms * bps;
                plan->nblocks = (int)std::max<long long>(
                    1, std::min<long long>(slots, (ncell + plan->nthreads - 1) / plan->nthreads));
            } else {
                cudaGetLastError();
            }
            // Face pass for nonlinear-Laplacian terms: each face is evaluated once per stage
            // instead of once for each of the two cells sharing it.  An extra launch per stage,
            // so by default only from 32768 cells on; MOL_FACE_PASS=0/1 forces it off/on.
            for (int k = 0; k < d->nterms; ++k)
                if (d->terms[k].kind == MOL_TERM_NONLINLAP) ++plan->nface;
            const char* fp = getenv("MOL_FACE_PASS");
            plan->face_pass = plan->nface > 0 && (fp && fp[0] ? fp[0] == '1' : ncell >= 32768);
            if (plan->face_pass && plan->jit.faces64) {
                // as many resident CTAs per SM as the face kernel's registers allow (MOL_FACE_CTAS
                // caps it): its loads and stores need the warps to hide their latency
                int bps = 0;
                if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void*)plan->jit.faces64, 256, 0) !=
                    cudaSuccess)
                    cudaGetLastError();
                if (const char* fc = getenv("MOL_FACE_CTAS"))
                    if (atoi(fc) > 0) bps = std::min(bps, atoi(fc));
                if (bps > 0) {
                    plan->face_threads = 256;
                    plan->face_blocks = (int)std::max<long long>(
                        1, std::min<long long>((long long)sms * bps, (ncell + 255) / 256));
                }
            }
        }
        // Coefficient stencils: the per-cell weights of the generated cell's variable groups,
        // once per plan (aux arrays are fixed at creation).  The face pass then serves only
        // terms outside the groups, and is dropped when there are none.
        if (plan->use_jit) {
            const std::vector<FoldGroup> groups = const_linear_groups(d);
            const int narr = fold_coef_arrays(groups);
            if (narr > 0) {
                if (!plan->jit.coef64) return fail(set_err(plan, MOL_ERR_CUDA, "coefficient kernel not loaded"));
                const size_t cells = (size_t)narr * (size_t)ncell;
                if ((st = plan_alloc(plan, (void**)&plan->coef64, sizeof(double) * cells))) return fail(st);
                if ((st = plan_alloc(plan, (void**)&plan->coef32, sizeof(float) * cells))) return fail(st);
                plan->ncoef = narr;
                const int grid = grid_for(ncell, sms, 4);
                cudaError_t e = launch_k(plan->jit.coef64, grid, kThreads, plan->stream, plan->P64, plan->coef64,
                                         plan->coef32);
                if (e == cudaSuccess) e = cudaStreamSynchronize(plan->stream);
                if ((st = cuda_check(plan, e, "coefficient stencils"))) return fail(st);
                ++g_launches;
                plan->P64.cw = plan->coef64;
                plan->P32.cw = plan->coef32;
                const char* fp = getenv("MOL_FACE_PASS");
                if (nonlinlap_all_in_groups(d, groups) && !(fp && fp[0] == '1')) plan->face_pass = false;
            }
        }
        if (!plan->use_jit) {
            const char* req = getenv("MOL_REQUIRE_CODEGEN");
            if (req && req[0] == '1') return fail(set_err(plan, st ? st : MOL_ERR_UNSUPPORTED, plan->jit_err));
        }
    }
    // Slabs of the streamed host-to-device copy: a stencil of any operator (its interior
    // taps, boundary and extrapolation tables) or a WENO term reaches at most `halo` slices
    // of the slowest dimension.  Only problems large enough to matter and with at least
    // 2 * halo + 1 slices per slab stream their state.
    {
        const int D = d->ndim - 1;
        long long reach = 2;
        for (int i = 0; i < d->nops; ++i) {
            const mol_op1d& o = d->ops[i];
            reach = std::max<long long>(reach, std::max({std::abs(o.omin), std::abs(o.omin + o.L - 1), o.bLlo, o.bLhi}));
        }
        plan->halo = reach + 1;
        for (int f = 0; f < d->nfields; ++f) plan->per_last |= d->bc[f][D][0].kind == MOL_BC_PERIODIC;
        const long long nsl = d->npts[D] - d->lower[D] - d->upper[D];
        const long long k = std::min<long long>(kMaxSlabs, nsl / (2 * plan->halo + 1));
        plan->h2d_slabs = (plan->ncell >= (1ll << 16) && k >= 2) ? (int)k : 0;
    }
    *out = plan;
    return MOL_OK;
}

// ----------------------------------------------------------------------------
// host/device staging
// ----------------------------------------------------------------------------

namespace {

template <class T>
struct Staged {
    T* ptr = nullptr;
    bool host = false;
};

template <class T>
int stage_in(mol_plan* plan, const T* src, int slot, Staged<T>& s, bool copy) {
    if (is_device_ptr(src)) {
        s.ptr = const_cast<T*>(src);
        s.host = false;
        return MOL_OK;
    }
    int st = ensure_slot<T>(plan, slot);
    if (st) return st;
    s.ptr = workspace<T>(plan)[slot];
    s.host = true;
    if (copy)
        return cuda_check(plan, cudaMemcpyAsync(s.ptr, src, sizeof(T) * (size_t)plan->nunk, cudaMemcpyHostToDevice,
                                                plan->stream), "H2D");
    return MOL_OK;
}

template <class T>
const T* params_ptr(mol_plan* plan, const T* p, int* st) {
    *st = MOL_OK;
    PlanArrays& A = std::is_same<T, double>::value ? plan->a64 : plan->a32;
    if (!p) return (const T*)A.params;
    if (is_device_ptr(p)) return p;
    const int np = std::max(plan->nparams, 0);
    bool same = A.params_known && (int)A.params_host.size() == np;
    for (int i = 0; same && i < np; ++i) same = (double)p[i] == A.params_host[i];
    if (same) return (const T*)A.params;
    *st = cuda_check(plan, cudaMemcpyAsync(A.params, p, sizeof(T) * (size_t)np, cudaMemcpyHostToDevice, plan->stream),
                     "params H2D");
    A.params_host.assign(p, p + np);
    A.params_known = !*st;
    return (const T*)A.params;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

template <class T>
int rhs_impl(mol_plan* plan, T* du, const T* u, const T* p, double t) {
    if (!plan || !du || !u || !std::isfinite(t)) return MOL_ERR_INVALID;
    DeviceGuard g(plan->dev);
    int st;
    // slots 10 and 11 stage host buffers for f!
    Staged<T> su, sdu;
    if ((st = stage_in<T>(plan, u, 10, su, true))) return st;
    if ((st = stage_in<T>(plan, du, 11, sdu, false))) return st;
    const T* pp = params_ptr<T>(plan, p, &st);
    if (st) return st;
    if ((st = ensure_faces<T>(plan))) return st;
    if ((st = launch_rhs<T>(plan, sdu.ptr, su.ptr, pp, t))) return st;
    if (sdu.host) {
        if ((st = cuda_check(plan, cudaMemcpyAsync(du, sdu.ptr, sizeof(T) * (size_t)plan->nunk, cudaMemcpyDeviceToHost,
                                                   plan->stream), "D2H")))
            return st;
        return cuda_check(plan, cudaStreamSynchronize(plan->stream), "sync");
    }
    return MOL_OK;
}

}  // namespace

// Waits for the plan's stream, then reports (and clears) the flag the last SSPRK33 stage sets
// when a step produced a NaN or Inf: OrdinaryDiffEq's unstable_check ending a solve.
int mol::sync_and_check_finite(mol_plan* plan) {
    int st = cuda_check(plan, cudaStreamSynchronize(plan->stream), "sync");
    if (st) return st;
    int bad = 0;
    if ((st = cuda_check(plan, cudaMemcpy(&bad, &plan->d_state->nonfinite, sizeof(int), cudaMemcpyDeviceToHost),
                         "status")))
        return st;
    if (!bad) return MOL_OK;
    cudaMemset(&plan->d_state->nonfinite, 0, sizeof(int));
    return set_err(plan, MOL_ERR_NONFINITE, "a step produced a NaN or Inf state value (unstable)");
}

namespace {

template <class T>
int ssprk_impl(mol_plan* plan, T* u, const T* p, double t0, double dt, int64_t nsteps) {
    if (!plan || !u || nsteps < 0 || !std::isfinite(dt) || !std::isfinite(t0)) return MOL_ERR_INVALID;
    DeviceGuard g(plan->dev);
    int st;
    if ((st = ensure_ws<T>(plan, 3))) return st;
    if ((st = ensure_faces<T>(plan))) return st;
    T** ws = workspace<T>(plan);
    Staged<T> su;
    const bool host = !is_device_ptr(u);
    T* ud = host ? ws[0] : u;
    // Pinned host state: the last stage writes the result straight into it over the coherent
    // host link instead of a bulk copy after the steps (stores do not stall the SMs, so the
    // write-back hides under the FP64-bound stage; reading the input that way measured slower
    // than the bulk copy, whose loads would stall).  MOL_ZERO_COPY=0 keeps both copies.
    T* hz = nullptr;
    if (host && nsteps > 0) {
        const char* zc = getenv("MOL_ZERO_COPY");
        if (!(zc && zc[0] == '0')) hz = (T*)mapped_host_ptr(u);
    }
    // Pinned host state and a problem that slabs along its slowest dimension: the first step's
    // stage 1 runs slab by slab behind the host-to-device copy (launch_stage1_streamed).
    // MOL_H2D_SLABS=0 copies first, then steps.
    int slabs = 0;
    if (host && nsteps > 0 && plan->h2d_slabs >= 2 && !face_pass_on<T>(plan) && mapped_host_ptr(u)) {
        const char* hs = getenv("MOL_H2D_SLABS");  // a slab count (0: copy first, then step)
        slabs = std::min(plan->h2d_slabs, (hs && hs[0]) ? std::max(0, atoi(hs)) : 4);
    }
    const bool streamed = slabs >= 2;
    if (host && !streamed &&
        (st = cuda_check(plan, cudaMemcpyAsync(ud, u, sizeof(T) * (size_t)plan->nunk, cudaMemcpyHostToDevice,
                                               plan->stream), "H2D")))
        return st;
    const T* pp = params_ptr<T>(plan, p, &st);
    if (st) return st;
    if (plan->use_jit) {  // modules are loaded before any stream capture begins
        st = ensure_fwd<T>(plan);
        if (st) return st;
    }
    k_set_time<<<1, 1, 0, plan->stream>>>(plan->d_state, t0);
    ++g_launches;
    T* u1 = ws[1];
    T* u2 = ws[2];
    if (streamed) {
        if ((st = launch_stage1_streamed<T>(plan, u, ud, u1, pp, dt, slabs))) return st;
        T* out1 = (nsteps == 1 && hz) ? hz : ud;
        if ((st = launch_ssprk_step_io<T>(plan, ud, out1, u1, u2, pp, dt, true))) return st;
        --nsteps;
        if (nsteps == 0 && hz) return sync_and_check_finite(plan);
    }
    if (nsteps == 0) hz = nullptr;  // nothing left to step: the state goes back by copy below
    const int64_t nmid = hz ? nsteps - 1 : nsteps;  // steps that stay in the device buffer ud
    // chunks of `chunk` steps replayed as one CUDA graph; the tail is launched directly
    const int chunk = plan->g_chunk;
    const bool is64 = std::is_same<T, double>::value;
    cudaGraphExec_t& gx = is64 ? plan->g_ssp64 : plan->g_ssp32;
    double& gdt = is64 ? plan->g_ssp64_dt : plan->g_ssp32_dt;
    const void*& gp = is64 ? plan->g_ssp64_p : plan->g_ssp32_p;
    const void*& gpp = is64 ? plan->g_ssp64_pp : plan->g_ssp32_pp;
    int64_t done = 0;
    // the legacy default stream cannot be captured: launch directly there
    const bool can_capture = plan->stream != nullptr && plan->stream != cudaStreamLegacy;
    if (nmid >= chunk && can_capture) {
        // the state buffer, parameter pointer and dt are baked into the captured graph
        if (gx && (gdt != dt || gp != (const void*)ud || gpp != (const void*)pp)) {
            cudaGraphExecDestroy(gx);
            gx = nullptr;
        }
        if (!gx) {
            cudaGraph_t graph;
            if ((st = cuda_check(plan, cudaStreamBeginCapture(plan->stream, cudaStreamCaptureModeThreadLocal),
                                 "capture")))
                return st;
            const long long before = g_launches.load();
            for (int s = 0; s < chunk; ++s) launch_ssprk_step<T>(plan, ud, u1, u2, pp, dt);
            g_launches = before;
            if ((st = cuda_check(plan, cudaStreamEndCapture(plan->stream, &graph), "end capture"))) return st;
            st = cuda_check(plan, cudaGraphInstantiate(&gx, graph, 0), "instantiate");
            cudaGraphDestroy(graph);
            if (st) return st;
            gdt = dt;
            gp = (const void*)ud;
            gpp = (const void*)pp;
        }
        for (; done + chunk <= nmid; done += chunk) {
            if ((st = cuda_check(plan, cudaGraphLaunch(gx, plan->stream), "graph launch"))) return st;
            g_launches += 3 * chunk;
        }
    }
    for (; done < nmid; ++done)
        if ((st = launch_ssprk_step<T>(plan, ud, u1, u2, pp, dt))) return st;
    if (hz) {
        if ((st = launch_ssprk_step_io<T>(plan, ud, hz, u1, u2, pp, dt))) return st;
        return sync_and_check_finite(plan);
    }
    if (host) {
        if ((st = cuda_check(plan, cudaMemcpyAsync(u, ud, sizeof(T) * (size_t)plan->nunk, cudaMemcpyDeviceToHost,
                                                   plan->stream), "D2H")))
            return st;
        return sync_and_check_finite(plan);
    }
    // device state: the call stays asynchronous; mol_plan_check reports a non-finite result
    return cuda_check(plan, cudaGetLastError(), "ssprk33");
}

}  // namespace

extern "C" {

int mol_fill_grid(mol_plan* plan, const double* u, const double* p, double t, double* full) {
    if (!plan || !u || !full || !std::isfinite(t)) return MOL_ERR_INVALID;
    DeviceGuard g(plan->dev);
    int st;
    Staged<double> su;
    if ((st = stage_in<double>(plan, u, 10, su, true))) return st;
    const double* pp = params_ptr<double>(plan, p, &st);
    if (st) return st;
    long long per_field = 1;
    for (int q = 0; q < plan->desc.ndim; ++q) per_field *= plan->desc.npts[q];
    const long long total = per_field * plan->nfields;
    const bool host = !is_device_ptr(full);
    double* out = full;
    if (host) {
        if (plan->grid_cap < total) {
            void* q = nullptr;
            if ((st = plan_alloc(plan, &q, sizeof(double) * (size_t)total))) return st;
            plan->grid_buf = (double*)q;
            plan->grid_cap = total;
        }
        out = plan->grid_buf;
    }
    const long long blocks = std::min<long long>((total + kThreads - 1) / kThreads, (long long)plan->sms * 8);
    k_fill_grid_t<double><<<(unsigned)std::max<long long>(blocks, 1), kThreads, 0, plan->stream>>>(
        plan->P64, su.ptr, pp, t, out, per_field);
    if ((st = cuda_check(plan, cudaGetLastError(), "fill_grid"))) return st;
    if (host) {
        if ((st = cuda_check(plan, cudaMemcpyAsync(full, out, sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost,
                                                   plan->stream), "D2H")))
            return st;
        return cuda_check(plan, cudaStreamSynchronize(plan->stream), "sync");
    }
    return MOL_OK;
}

int mol_rhs(mol_plan* plan, double* du, const double* u, const double* p, double t) {
    return rhs_impl<double>(plan, du, u, p, t);
}
int mol_rhs_f32state(mol_plan* plan, float* du, const float* u, const float* p, double t) {
    return rhs_impl<float>(plan, du, u, p, t);
}
int mol_step_ssprk33(mol_plan* plan, double* u, const double* p, double t0, double dt, int64_t nsteps) {
    return ssprk_impl<double>(plan, u, p, t0, dt, nsteps);
}
int mol_step_ssprk33_f32state(mol_plan* plan, float* u, const float* p, double t0, double dt, int64_t nsteps) {
    return ssprk_impl<float>(plan, u, p, t0, dt, nsteps);
}
int mol_plan_check(mol_plan* plan) {
    if (!plan) return MOL_ERR_INVALID;
    DeviceGuard g(plan->dev);
    return sync_and_check_finite(plan);
}

}  // extern "C"

namespace {

// End of a Tsit5 solve: statistics, the state back to host memory, the controller's status.
int tsit_finish(mol_plan* plan, double* u, const double* ud, bool host, const SolverState& hs, mol_stats* stats) {
    int st;
    if (stats) {
        stats->naccept = hs.naccept;
        stats->nreject = hs.nreject;
        stats->nf = hs.nf + 1;
        stats->t = hs.t;
        stats->dt = hs.dt;
    }
    if (host) {
        if ((st = cuda_check(plan, cudaMemcpyAsync(u, ud, sizeof(double) * (size_t)plan->nunk, cudaMemcpyDeviceToHost,
                                                   plan->stream), "D2H")))
            return st;
        if ((st = cuda_check(plan, cudaStreamSynchronize(plan->stream), "sync"))) return st;
    }
    if (hs.status) return set_err(plan, hs.status, "tsit5 stopped early");
    return MOL_OK;
}

}  // namespace

extern "C" {

int mol_solve_tsit5(mol_plan* plan, double* u, const double* p, double t0, double t1, double abstol, double reltol,
                    double dt0, int64_t maxiters, mol_stats* stats) {
    if (!plan || !u || !std::isfinite(t0) || !std::isfinite(t1) || !(t1 >= t0) || !(abstol > 0) ||
        !std::isfinite(abstol) || !(reltol >= 0) || !std::isfinite(reltol) || !std::isfinite(dt0))
        return MOL_ERR_INVALID;
    DeviceGuard g(plan->dev);
    int st;
    // slots: 0 u, 1..7 k1..k7, 8 ybuf0, 9 ybuf1
    if ((st = ensure_ws<double>(plan, 10))) return st;
    double** ws = plan->ws64;
    const bool host = !is_device_ptr(u);
    double* ud = host ? ws[0] : u;
    if (host && (st = cuda_check(plan, cudaMemcpyAsync(ud, u, sizeof(double) * (size_t)plan->nunk,
                                                       cudaMemcpyHostToDevice, plan->stream), "H2D")))
        return st;
    const double* pp = params_ptr<double>(plan, p, &st);
    if (st) return st;
    double** d_k = nullptr;
    {
        void* tmp;
        if ((st = plan_alloc(plan, &tmp, sizeof(double*) * 7))) return st;
        d_k = (double**)tmp;
        double* hk[7];
        for (int i = 0; i < 7; ++i) hk[i] = ws[1 + i];
        if ((st = cuda_check(plan, cudaMemcpyAsync(d_k, hk, sizeof(hk), cudaMemcpyHostToDevice, plan->stream), "k ptrs")))
            return st;
    }
    const long long n = plan->nunk;
    double* k1 = ws[1];
    double* k7 = ws[7];
    double* yb0 = ws[8];
    double* yb1 = ws[9];
    const int nb = plan->nblocks;
    // k1 = f(u0, t0)
    if ((st = launch_rhs<double>(plan, k1, ud, pp, t0))) return st;
    double dt = dt0;
    if (!(dt > 0)) {
        // Hairer's initial step (the heuristic OrdinaryDiffEq's ode_determine_initdt follows)
        std::vector<double> hp(3 * nb);
        k_init_norms<double><<<nb, kThreads, 0, plan->stream>>>(n, ud, k1, nullptr, abstol, reltol, plan->d_partials);
        ++g_launches;
        cudaMemcpyAsync(hp.data(), plan->d_partials, sizeof(double) * 3 * nb, cudaMemcpyDeviceToHost, plan->stream);
        if ((st = cuda_check(plan, cudaStreamSynchronize(plan->stream), "init norms"))) return st;
        double s0 = 0, s1 = 0;
        for (int b = 0; b < nb; ++b) { s0 += hp[3 * b]; s1 += hp[3 * b + 1]; }
        const double d0 = std::sqrt(s0 / n), d1 = std::sqrt(s1 / n);
        double h0 = (d0 < 1e-5 || d1 < 1e-5) ? 1e-6 : 0.01 * d0 / d1;
        h0 = std::min(h0, t1 - t0);
        k_axpy<double><<<nb, kThreads, 0, plan->stream>>>(n, yb1, ud, k1, h0);
        ++g_launches;
        if ((st = launch_rhs<double>(plan, yb0, yb1, pp, t0 + h0))) return st;
        k_init_norms<double><<<nb, kThreads, 0, plan->stream>>>(n, ud, k1, yb0, abstol, reltol, plan->d_partials);
        ++g_launches;
        cudaMemcpyAsync(hp.data(), plan->d_partials, sizeof(double) * 3 * nb, cudaMemcpyDeviceToHost, plan->stream);
        if ((st = cuda_check(plan, cudaStreamSynchronize(plan->stream), "init norms"))) return st;
        double s2 = 0;
        for (int b = 0; b < nb; ++b) s2 += hp[3 * b + 2];
        const double d2 = std::sqrt(s2 / n) / h0;
        const double m = std::max(d1, d2);
        const double h1 = m <= 1e-15 ? std::max(1e-6, h0 * 1e-3) : std::pow(0.01 / m, 1.0 / 5.0);
        dt = std::min(std::min(100 * h0, h1), t1 - t0);
    }
    if (maxiters <= 0) maxiters = 100000000;
    k_tsit_init_state<<<1, 1, 0, plan->stream>>>(plan->d_state, t0, t1, dt, abstol, reltol, maxiters);
    ++g_launches;
    k_tsit_commit<double><<<nb, kThreads, 0, plan->stream>>>(plan->P64, ud, k1, k7, yb1, yb0, plan->d_state, 1);
    ++g_launches;
    // Small problems: one CTA runs whole attempts (k_tsit_small_t), kSmallAttempts per launch,
    // instead of seven launches per attempt.  Measured threshold: below about a thousand
    // unknowns an attempt's launches cost more than its arithmetic on one SM.
    constexpr long long kSmallTsit = 1024;
    constexpr long long kSmallTsitShared = 512;   // 10 arrays of 8 bytes in 40 KB of shared memory
    constexpr int kSmallAttempts = 256;
    if (plan->use_jit && plan->jit.tsitsmall64 && n <= kSmallTsit && !getenv("MOL_TSIT_NO_SMALL")) {
        SolverState hs;
        const int smem = n <= kSmallTsitShared ? 1 : 0;
        const size_t bytes = smem ? sizeof(double) * 10 * (size_t)n : 0;
        for (;;) {
            if ((st = cuda_check(plan, launch_ks(plan->jit.tsitsmall64, 1, kThreads, bytes, plan->stream, plan->P64,
                                                 ud, (double* const*)d_k, yb0, yb1, pp, plan->d_state,
                                                 kSmallAttempts, smem),
                                 "tsit5 small launch")))
                return st;
            ++g_launches;
            cudaMemcpyAsync(&hs, plan->d_state, sizeof(SolverState), cudaMemcpyDeviceToHost, plan->stream);
            if ((st = cuda_check(plan, cudaStreamSynchronize(plan->stream), "tsit5 sync"))) return st;
            if (hs.done) break;
        }
        return tsit_finish(plan, u, ud, host, hs, stats);
    }
    // one attempt = stages 2..7 + commit; M attempts per captured graph
    auto attempt = [&]() {
        for (int s = 2; s <= 7; ++s) {
            const double* yin = (s % 2 == 0) ? yb0 : yb1;
            double* yout = (s % 2 == 0) ? yb1 : yb0;
            if (plan->use_jit)
                launch_k(plan->jit.tsit64, nb, plan->nthreads, plan->stream, plan->P64, s, yin, yout, (const double*)ud,
                         (double* const*)d_k, pp, plan->d_state, plan->d_partials);
            else
                k_tsit_stage_t<double, InterpCell><<<nb, kThreads, 0, plan->stream>>>(
                    plan->P64, s, yin, yout, ud, d_k, pp, plan->d_state, plan->d_partials);
        }
        k_tsit_commit<double><<<nb, kThreads, 0, plan->stream>>>(plan->P64, ud, k1, k7, yb1, yb0, plan->d_state, 0);
    };
    const int M = 32;
    cudaGraph_t graph;
    cudaGraphExec_t gx = nullptr;
    const bool can_capture = plan->stream != nullptr && plan->stream != cudaStreamLegacy;
    if (can_capture) {
        if ((st = cuda_check(plan, cudaStreamBeginCapture(plan->stream, cudaStreamCaptureModeThreadLocal),
                             "capture")))
            return st;
        for (int i = 0; i < M; ++i) attempt();
        if ((st = cuda_check(plan, cudaStreamEndCapture(plan->stream, &graph), "end capture"))) return st;
        st = cuda_check(plan, cudaGraphInstantiate(&gx, graph, 0), "instantiate");
        cudaGraphDestroy(graph);
        if (st) return st;
    }
    SolverState hs;
    for (;;) {
        if (can_capture) {
            if ((st = cuda_check(plan, cudaGraphLaunch(gx, plan->stream), "graph launch"))) break;
        } else {
            for (int i = 0; i < M; ++i) attempt();
            if ((st = cuda_check(plan, cudaGetLastError(), "tsit5 launch"))) break;
        }
        g_launches += 7 * M;
        cudaMemcpyAsync(&hs, plan->d_state, sizeof(SolverState), cudaMemcpyDeviceToHost, plan->stream);
        if ((st = cuda_check(plan, cudaStreamSynchronize(plan->stream), "tsit5 sync"))) break;
        if (hs.done) break;
    }
    if (gx) cudaGraphExecDestroy(gx);
    if (st) return st;
    return tsit_finish(plan, u, ud, host, hs, stats);
}

}  // extern "C"
