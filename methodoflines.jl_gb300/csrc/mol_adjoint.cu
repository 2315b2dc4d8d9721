// Discrete adjoint of fixed-step SSPRK33 with binomial checkpointing.
//
// The reference has no adjoint of its own (gradients of a MethodOfLines solve
// come from generic AD through OrdinaryDiffEq); this is the hand-written
// reverse sweep of the exact discrete map the GPU integrates:
//   u1 = u + dt f(u, t)
//   u2 = (3u + u1 + dt f(u1, t+dt)) / 4
//   u' = (u + 2 u2 + 2 dt f(u2, t+dt/2)) / 3
// Reverse, given lam = dL/du':
//   l2 = 2/3 lam + 2dt/3 J(u2)^T lam
//   l1 = 1/4 l2  + dt/4  J(u1)^T l2
//   lam_u = 1/3 lam + 3/4 l2 + l1 + dt J(u)^T l1
// with the same scaled products accumulated into dL/dp and dL/daux.  The
// vector-Jacobian products are the generated reverse sweep of f (mol_codegen.cu).
// With the three products kept in accumulators
//   C = 2dt/3 J(u2)^T lam,  A1 = dt/4 J(u1)^T l2,  A0 = dt J(u)^T l1
// the combinations become l2 = 2/3 lam + C, l1 = 1/6 lam + 1/4 C + A1 and
// lam_u = lam + C + A1 + A0.  Each VJP launch reads its seed as such a combination
// (k_vjp_t's VjpSeed), and the first launch of the next reverse step folds the
// previous step's accumulators into lam and clears them, so a reverse step is two
// stage recomputations and three VJP launches with no separate combination pass.
// C alternates between two buffers so the launch accumulating the new C never
// shares a buffer with the one it folds.
// States between checkpoints are recomputed; checkpoint positions follow the
// binomial (revolve) schedule of Griewank & Walther for `nsnap` slots (mol_schedule.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "mol_kernels.cuh"
#include "mol_plan.h"
#include "mol_schedule.h"

namespace mol {

namespace {

__global__ void k_lincomb3(long long n, double* out, double a, const double* x, double b, const double* y, double c,
                           const double* z) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        double v = a * x[g];
        if (y) v = fma(b, y[g], v);
        if (z) v = fma(c, z[g], v);
        out[g] = v;
    }
}

// out = u - target and per-block partial sums of (u - target)^2.
__global__ void k_misfit(long long n, const double* u, const double* target, double* out, double* partials) {
    double s = 0.0;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x) {
        const double r = u[g] - target[g];
        out[g] = r;
        s = fma(r, r, s);
    }
    __shared__ double red[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) t += red[w];
        partials[blockIdx.x] = t;
    }
}

struct Adj {
    mol_plan* plan;
    long long n;
    int nb;
    double dt, t0;
    const double* p;
    double* target;
    int loss_kind;
    int64_t N;
    // buffers
    std::vector<double*> slots;
    double *work, *u1, *u2, *lam, *cbuf[2], *a1, *a0, *tmp;
    int cur = 0;                 // cbuf[cur] holds C of the latest reverse step
    double* lam_p;
    double* lam_aux;
    bool have_lam = false;
    double loss = 0.0;
    double* uT_dev = nullptr;
    long long fwd_steps = 0;
    int err = MOL_OK;
    // Launches are recorded into CUDA graphs of about kGraphLaunches kernels and replayed
    // once each: a reverse step is five short launches, and on small grids the gaps
    // between stream launches would otherwise cost as much as the kernels.
    static constexpr int kGraphLaunches = 240;
    bool graphs = false;
    bool capturing = false;
    int pending = 0;
    std::vector<cudaGraphExec_t> execs;

    int ck(cudaError_t e, const char* w) {
        if (err) return err;
        err = cuda_check(plan, e, w);
        return err;
    }

    void cap_begin() {
        if (!graphs || capturing || err) return;
        cudaError_t e = cudaStreamBeginCapture(plan->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaGetLastError();
            graphs = false;
            return;
        }
        capturing = true;
        pending = 0;
    }

    void cap_end() {
        if (!capturing) return;
        capturing = false;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(plan->stream, &g);
        if (e != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            ck(e != cudaSuccess ? e : cudaErrorStreamCaptureInvalidated, "adjoint capture");
            return;
        }
        cudaGraphExec_t x = nullptr;
        e = cudaGraphInstantiate(&x, g, 0);
        cudaGraphDestroy(g);
        if (ck(e, "adjoint graph instantiate")) return;
        execs.push_back(x);
        ck(cudaGraphLaunch(x, plan->stream), "adjoint graph launch");
    }

    void counted() {
        if (capturing && ++pending >= kGraphLaunches) cap_end();
    }

    void release_graphs() {
        for (cudaGraphExec_t x : execs) cudaGraphExecDestroy(x);
        execs.clear();
    }

    double time_of(int64_t m) const { return t0 + (double)m * dt; }

    void stage(int which, const double* uin, const double* u0, double* uout, double t) {
        if (err) return;
        const double* cu = uin;
        cap_begin();
        // the stage's time offset, as the stage kernel forms it from t
        const double toff = which == 1 ? 0.0 : (which == 2 ? dt : dt / 2);
        cudaError_t e;
        const DevProb<double> P = with_faces<double>(plan, cu, p, toff, t, &e);
        if (e == cudaSuccess)
            e = launch_k(plan->jit.ssp64[which - 1], plan->nblocks, plan->nthreads, plan->stream, P, cu, u0, uout, p,
                         plan->d_state, which == 3 ? 2 * dt : dt, t, 0ll, (long long)plan->ncell);
        ++g_launches;
        ck(e, "stage launch");
        counted();
    }

    // state at step `from` in src -> state at step `from + k` in dst; the first step
    // writes dst directly, later ones update it in place.  Stage times are t0 + m dt.
    void advance(const double* src, double* dst, int64_t from, int64_t k) {
        if (err) return;
        if (k == 0) {
            if (dst != src)
                ck(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, plan->stream), "copy");
            return;
        }
        const double* in = src;
        for (int64_t s = 0; s < k && !err; ++s) {
            const double tm = time_of(from + s);
            stage(1, in, in, u1, tm);
            stage(2, u1, in, u2, tm);
            stage(3, u2, in, dst, tm);
            in = dst;
        }
        fwd_steps += k;
    }

    void vjp(const VjpSeed<double>& in, double scale, const double* u, double t, double* out) {
        if (err) return;
        const DevProb<double>& P = plan->P64;
        cap_begin();
        cudaError_t e = launch_k(plan->jit.vjp64, plan->vjp_blocks > 0 ? plan->vjp_blocks : plan->nblocks, plan->nthreads, plan->stream, P, in, scale, u, p, t,
                                 out, lam_p, lam_aux);
        ++g_launches;
        ck(e, "vjp launch");
        counted();
    }

    // Reverse step m, the state u_m being in `um`: its stage values are recomputed.
    void reverse_step(const double* um, int64_t m) {
        if (err) return;
        const double tm = time_of(m);
        stage(1, um, um, u1, tm);
        stage(2, u1, um, u2, tm);
        fwd_steps += 1;
        if (!have_lam) {
            // last step: u_N and dL/du_N
            stage(3, u2, um, tmp, tm);
            start_lambda(tmp);
        }
        reverse_vjps(um, u1, u2, tm);
    }

    // u_N is in uN: the loss, and dL/du_N into lam.
    void start_lambda(const double* uN) {
        if (err) return;
        {
            if (uT_dev) ck(cudaMemcpyAsync(uT_dev, uN, sizeof(double) * n, cudaMemcpyDeviceToDevice, plan->stream), "uT");
            if (loss_kind == MOL_LOSS_MISFIT) {
                k_misfit<<<nb, kThreads, 0, plan->stream>>>(n, uN, target, lam, plan->d_partials);
                ++g_launches;
                cap_end();  // the loss is read on the host here
                std::vector<double> hp(nb);
                ck(cudaMemcpyAsync(hp.data(), plan->d_partials, sizeof(double) * nb, cudaMemcpyDeviceToHost,
                                   plan->stream), "loss");
                ck(cudaStreamSynchronize(plan->stream), "loss sync");
                double s = 0.0;
                for (double v : hp) s += v;
                loss = 0.5 * s;
            } else {
                ck(cudaMemcpyAsync(lam, target, sizeof(double) * n, cudaMemcpyDeviceToDevice, plan->stream), "lambda");
            }
            have_lam = true;
        }
    }

    // The three VJP launches of reverse step m given u_m and its stage values u1, u2.
    void reverse_vjps(const double* um, const double* su1, const double* su2, double tm) {
        if (err) return;
        double* Cold = cbuf[cur];
        double* Cnew = cbuf[cur ^ 1];
        cur ^= 1;
        // lam <- lam + C + A1 + A0 of the step before (all zero before the first), then
        // Cnew = 2dt/3 J(u2)^T lam
        VjpSeed<double> s2 = {};
        s2.x[0] = lam; s2.x[1] = Cold; s2.x[2] = a1; s2.x[3] = a0;
        s2.a[0] = s2.a[1] = s2.a[2] = s2.a[3] = 1.0;
        s2.upd = lam;
        s2.zero[0] = Cold; s2.zero[1] = a1; s2.zero[2] = a0;
        vjp(s2, 2.0 * dt / 3.0, su2, tm + dt / 2, Cnew);
        // A1 = dt/4 J(u1)^T l2,  l2 = 2/3 lam + C
        VjpSeed<double> s1 = {};
        s1.x[0] = lam; s1.x[1] = Cnew;
        s1.a[0] = 2.0 / 3.0; s1.a[1] = 1.0;
        vjp(s1, dt / 4.0, su1, tm + dt, a1);
        // A0 = dt J(u)^T l1,  l1 = 1/6 lam + 1/4 C + A1
        VjpSeed<double> s0 = {};
        s0.x[0] = lam; s0.x[1] = Cnew; s0.x[2] = a1;
        s0.a[0] = 1.0 / 6.0; s0.a[1] = 0.25; s0.a[2] = 1.0;
        vjp(s0, dt, um, tm, a0);
    }

    // Everything kept: states S[0..N] and the stage values U1[m], U2[m] of every step, so
    // the reverse sweep is the three VJP launches per step and nothing is recomputed
    // (the GB300's HBM holds tens of thousands of states of a mid-size grid).
    void stored_sweep(double* const* S, double* const* U1, double* const* U2) {
        for (int64_t m = 0; m < N && !err; ++m) {
            const double tm = time_of(m);
            stage(1, S[m], S[m], U1[m], tm);
            stage(2, U1[m], S[m], U2[m], tm);
            stage(3, U2[m], S[m], S[m + 1], tm);
        }
        fwd_steps += N;
        cap_end();
        start_lambda(S[N]);
        for (int64_t m = N - 1; m >= 0 && !err; --m) reverse_vjps(S[m], U1[m], U2[m], time_of(m));
    }

    // dL/du_0 = lam + C + A1 + A0 of the last reverse step, into lam.
    void finish() {
        cap_end();
        if (err) return;
        k_lincomb3<<<nb, kThreads, 0, plan->stream>>>(n, lam, 1.0, lam, 1.0, cbuf[cur], 1.0, a1);
        k_lincomb3<<<nb, kThreads, 0, plan->stream>>>(n, lam, 1.0, lam, 1.0, a0, 0.0, nullptr);
        g_launches += 2;
        ck(cudaGetLastError(), "adjoint combine");
    }

    // Reverse steps [l, r) with the state u_l in slot `sl`; `free` are spare slots.
    void rev(int64_t l, int64_t r, double* sl, std::vector<double*>& free) {
        if (err || r <= l) return;
        if (r - l == 1) {
            reverse_step(sl, l);
            return;
        }
        if (free.empty()) {
            for (int64_t m = r - 1; m >= l && !err; --m) {
                if (m == l) {
                    reverse_step(sl, l);
                } else {
                    advance(sl, work, l, m - l);
                    reverse_step(work, m);
                }
            }
            return;
        }
        if ((int64_t)free.size() >= r - l - 1) {
            // every state of [l, r) has a slot: store them walking forward and reverse walking
            // back (the recursion would peel one step per level, as deep as the horizon)
            std::vector<double*> st(1, sl);
            for (int64_t k = l + 1; k < r && !err; ++k) {
                double* q = free.back();
                free.pop_back();
                advance(st.back(), q, k - 1, 1);
                st.push_back(q);
            }
            for (int64_t m = r - 1; m >= l && !err; --m) reverse_step(st[m - l], m);
            for (size_t i = 1; i < st.size(); ++i) free.push_back(st[i]);
            return;
        }
        const int64_t m = l + checkpoint_split(r - l, (int)free.size());
        double* sm = free.back();
        free.pop_back();
        advance(sl, sm, l, m - l);
        rev(m, r, sm, free);
        free.push_back(sm);
        rev(l, m, sl, free);
    }
};

__global__ void k_zero(long long n, double* x) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n; g += (long long)gridDim.x * blockDim.x)
        x[g] = 0.0;
}

}  // namespace

}  // namespace mol

using namespace mol;

namespace {

int need_vjp(mol_plan* plan) {
    if (!plan->use_jit)
        return set_err(plan, MOL_ERR_UNSUPPORTED,
                       "the vector-Jacobian product is generated code only (code generation is off: " + plan->jit_err + ")");
    if (plan->nparams > 16) return set_err(plan, MOL_ERR_UNSUPPORTED, "at most 16 parameters for the adjoint");
    int st = jit_ensure(&plan->jit, JIT_VJP, plan->jit_err);
    if (st) return set_err(plan, st, plan->jit_err);
    st = jit_ensure(&plan->jit, JIT_FWD64, plan->jit_err);
    if (st) return set_err(plan, st, plan->jit_err);
    if (!plan->vjp_blocks) {
        // SMs x the VJP kernel's resident CTAs (a grid-stride loop: one wave)
        int bps = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void*)plan->jit.vjp64, plan->nthreads, 0) !=
            cudaSuccess)
            cudaGetLastError();
        plan->vjp_blocks = bps > 0 ? (int)std::max<long long>(1, std::min<long long>((long long)plan->sms * bps,
                                                                   (plan->ncell + plan->nthreads - 1) / plan->nthreads))
                                   : plan->nblocks;
    }
    return MOL_OK;
}

// Copy host or device input into a device buffer (returns the device pointer to use).
const double* dev_in(mol_plan* plan, const double* src, double* scratch, size_t n, int* st) {
    *st = MOL_OK;
    if (!src) return nullptr;
    if (is_device_ptr(src)) return src;
    *st = cuda_check(plan, cudaMemcpyAsync(scratch, src, sizeof(double) * n, cudaMemcpyHostToDevice, plan->stream), "H2D");
    return scratch;
}

int dev_out(mol_plan* plan, double* dst, const double* src, size_t n) {
    if (!dst) return MOL_OK;
    return cuda_check(plan, cudaMemcpyAsync(dst, src, sizeof(double) * n,
                                            is_device_ptr(dst) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                            plan->stream), "D2H");
}

}  // namespace

extern "C" {

int mol_rhs_vjp(mol_plan* plan, const double* lambda, const double* u, const double* p, double t, double* lam_u,
                double* lam_p, double* lam_aux) {
    if (!plan || !lambda || !u) return MOL_ERR_INVALID;
    int st = need_vjp(plan);
    if (st) return st;
    const long long n = plan->nunk;
    double* A[6];
    for (int i = 0; i < 6; ++i) {
        if (!plan->adj[i]) {
            void* q;
            const size_t sz = i < 3 ? (size_t)n : (i == 3 ? (size_t)std::max(plan->nparams, 1)
                                                          : (size_t)std::max<long long>(plan->aux_total, 1));
            if ((st = plan_alloc(plan, &q, sizeof(double) * sz))) return st;
            plan->adj[i] = (double*)q;
        }
        A[i] = plan->adj[i];
    }
    const double* dl = dev_in(plan, lambda, A[0], n, &st);
    if (st) return st;
    const double* du = dev_in(plan, u, A[1], n, &st);
    if (st) return st;
    int pst = 0;
    const double* pp = p ? (is_device_ptr(p) ? p : nullptr) : (const double*)plan->a64.params;
    if (p && !pp) {
        plan->a64.params_known = false;
        pst = cuda_check(plan, cudaMemcpyAsync(plan->a64.params, p, sizeof(double) * plan->nparams,
                                               cudaMemcpyHostToDevice, plan->stream), "params");
        if (pst) return pst;
        pp = (const double*)plan->a64.params;
    }
    // outputs accumulate: start from the caller's values
    auto prep = [&](double* user, double* buf, size_t cnt) -> double* {
        if (!user) {
            k_zero<<<64, 256, 0, plan->stream>>>((long long)cnt, buf);
            return buf;
        }
        if (is_device_ptr(user)) return user;
        cudaMemcpyAsync(buf, user, sizeof(double) * cnt, cudaMemcpyHostToDevice, plan->stream);
        return buf;
    };
    double* ou = prep(lam_u, A[2], n);
    double* op = prep(lam_p, A[3], std::max(plan->nparams, 1));
    double* oa = lam_aux ? prep(lam_aux, A[4], std::max<long long>(plan->aux_total, 1)) : nullptr;
    const DevProb<double>& P = plan->P64;
    VjpSeed<double> in = {};
    in.x[0] = dl;
    in.a[0] = 1.0;
    cudaError_t e = launch_k(plan->jit.vjp64, plan->vjp_blocks > 0 ? plan->vjp_blocks : plan->nblocks, plan->nthreads, plan->stream, P, in, 1.0, du, pp, t, ou,
                             lam_p ? op : (double*)nullptr, oa);
    ++g_launches;
    if ((st = cuda_check(plan, e, "vjp"))) return st;
    if (lam_u && !is_device_ptr(lam_u) && (st = dev_out(plan, lam_u, ou, n))) return st;
    if (lam_p && !is_device_ptr(lam_p) && (st = dev_out(plan, lam_p, op, plan->nparams))) return st;
    if (lam_aux && !is_device_ptr(lam_aux) && (st = dev_out(plan, lam_aux, oa, plan->aux_total))) return st;
    return cuda_check(plan, cudaStreamSynchronize(plan->stream), "vjp sync");
}

int mol_adjoint_ssprk33(mol_plan* plan, const double* u0, const double* p, double t0, double dt, int64_t nsteps,
                        int32_t nsnap, int32_t loss_kind, const double* target, double* uT, double* loss,
                        double* dLdu0, double* dLdp, double* dLdaux, int64_t* nforward_steps) {
    if (!plan || !u0 || !target || nsteps < 0 || !(dt > 0) || !std::isfinite(dt) || !std::isfinite(t0) ||
        (loss_kind != MOL_LOSS_MISFIT && loss_kind != MOL_LOSS_LAMBDA))
        return MOL_ERR_INVALID;
    int st = need_vjp(plan);
    if (st) return st;
    if ((st = ensure_faces<double>(plan))) return st;
    const long long n = plan->nunk;
    // working buffers
    std::vector<void*> mine;
    auto get = [&](size_t cnt) -> double* {
        void* q = nullptr;
        if (cudaMalloc(&q, sizeof(double) * std::max<size_t>(cnt, 1)) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        mine.push_back(q);
        return (double*)q;
    };
    auto release = [&]() {
        cudaStreamSynchronize(plan->stream);
        for (void* q : mine) cudaFree(q);
    };
    // checkpoint slots.  nsnap <= 0: keep every state and both stage values of every step
    // when they fit in three quarters of the free memory (no recomputation at all), else as
    // many states as fit (binomial schedule over them).  The buffers live for the call only;
    // the quarter left is for the caller (the 400-step 256^3 ADR adjoint keeps 161 GB of its
    // 280 GB device this way instead of recomputing two stages per reverse step).
    constexpr double kAdjointMemFraction = 0.75;
    int64_t slots = nsnap;
    bool keep_stages = false;
    if (slots <= 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        keep_stages = nsteps > 0 && (3.0 * nsteps + 1.0) * 8.0 * n <= kAdjointMemFraction * fr;
        slots = (int64_t)std::max<double>(
            2.0, std::min<double>((double)nsteps + 1, kAdjointMemFraction * fr / (8.0 * n)));
    }
    slots = std::max<int64_t>(1, std::min<int64_t>(slots, nsteps + 1));
    Adj A;
    A.plan = plan;
    A.n = n;
    A.nb = plan->nblocks;
    A.dt = dt;
    A.t0 = t0;
    A.loss_kind = loss_kind;
    A.N = nsteps;
    {
        const char* g = getenv("MOL_ADJOINT_GRAPHS");
        A.graphs = plan->stream != nullptr && plan->stream != cudaStreamLegacy && !(g && g[0] == '0');
    }
    std::vector<double*> S1, S2;
    if (keep_stages) {
        double* all = get((size_t)(3 * nsteps + 1) * (size_t)n);
        if (!all) {
            keep_stages = false;
        } else {
            for (int64_t i = 0; i <= nsteps; ++i) A.slots.push_back(all + (size_t)i * n);
            for (int64_t i = 0; i < nsteps; ++i) {
                S1.push_back(all + (size_t)(nsteps + 1 + i) * n);
                S2.push_back(all + (size_t)(2 * nsteps + 1 + i) * n);
            }
        }
    }
    for (int64_t i = 0; !keep_stages && i < slots; ++i) {
        double* q = get(n);
        if (!q) {
            release();
            return set_err(plan, MOL_ERR_OOM, "checkpoint slots do not fit in device memory");
        }
        A.slots.push_back(q);
    }
    A.work = get(n);
    A.u1 = get(n);
    A.u2 = get(n);
    A.lam = get(n);
    A.cbuf[0] = get(n);
    A.cbuf[1] = get(n);
    A.a1 = get(n);
    A.a0 = get(n);
    A.tmp = get(n);
    A.target = get(n);
    A.lam_p = get(std::max(plan->nparams, 1));
    A.lam_aux = get((size_t)std::max<long long>(plan->aux_total, 1));
    double* pbuf = get(std::max(plan->nparams, 1));
    if (!A.work || !A.u1 || !A.u2 || !A.lam || !A.cbuf[0] || !A.cbuf[1] || !A.a1 || !A.a0 || !A.tmp || !A.target ||
        !A.lam_p || !A.lam_aux || !pbuf) {
        release();
        return set_err(plan, MOL_ERR_OOM, "adjoint buffers do not fit in device memory");
    }
    if (uT) A.uT_dev = get(n);
    // inputs
    const double* du0 = dev_in(plan, u0, A.slots[0], n, &st);
    if (!st && du0 != A.slots[0])
        st = cuda_check(plan, cudaMemcpyAsync(A.slots[0], du0, sizeof(double) * n, cudaMemcpyDeviceToDevice, plan->stream),
                        "u0");
    if (!st) {
        const double* dtg = dev_in(plan, target, A.target, n, &st);
        if (!st && dtg != A.target)
            st = cuda_check(plan, cudaMemcpyAsync(A.target, dtg, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                                  plan->stream), "target");
    }
    if (!st && p) st = cuda_check(plan, cudaMemcpyAsync(pbuf, p, sizeof(double) * plan->nparams,
                                                         is_device_ptr(p) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                                         plan->stream), "params");
    A.p = p ? pbuf : (const double*)plan->a64.params;
    if (st) {
        release();
        return st;
    }
    k_zero<<<64, 256, 0, plan->stream>>>(std::max(plan->nparams, 1), A.lam_p);
    k_zero<<<1024, 256, 0, plan->stream>>>(std::max<long long>(plan->aux_total, 1), A.lam_aux);
    for (double* q : {A.cbuf[0], A.cbuf[1], A.a1, A.a0}) k_zero<<<1024, 256, 0, plan->stream>>>(n, q);
    if (nsteps == 0) {
        // L depends on u0 directly
        if (loss_kind == MOL_LOSS_MISFIT) {
            k_misfit<<<A.nb, kThreads, 0, plan->stream>>>(n, A.slots[0], A.target, A.lam, plan->d_partials);
            std::vector<double> hp(A.nb);
            cudaMemcpyAsync(hp.data(), plan->d_partials, sizeof(double) * A.nb, cudaMemcpyDeviceToHost, plan->stream);
            cudaStreamSynchronize(plan->stream);
            for (double v : hp) A.loss += v;
            A.loss *= 0.5;
        } else {
            cudaMemcpyAsync(A.lam, A.target, sizeof(double) * n, cudaMemcpyDeviceToDevice, plan->stream);
        }
        if (A.uT_dev) cudaMemcpyAsync(A.uT_dev, A.slots[0], sizeof(double) * n, cudaMemcpyDeviceToDevice, plan->stream);
    } else {
        if (keep_stages) {
            A.stored_sweep(A.slots.data(), S1.data(), S2.data());
        } else {
            std::vector<double*> free(A.slots.begin() + 1, A.slots.end());
            A.rev(0, nsteps, A.slots[0], free);
        }
        A.finish();
    }
    A.cap_end();
    st = A.err;
    if (!st && uT) st = dev_out(plan, uT, A.uT_dev, n);
    if (!st && dLdu0) st = dev_out(plan, dLdu0, A.lam, n);
    if (!st && dLdp && plan->nparams > 0) st = dev_out(plan, dLdp, A.lam_p, plan->nparams);
    if (!st && dLdaux && plan->aux_total > 0) st = dev_out(plan, dLdaux, A.lam_aux, plan->aux_total);
    if (!st) st = cuda_check(plan, cudaStreamSynchronize(plan->stream), "adjoint sync");
    // a forward (re)computed step with a NaN or Inf state, or a non-finite misfit
    if (!st) st = sync_and_check_finite(plan);
    if (!st && !std::isfinite(A.loss))
        st = set_err(plan, MOL_ERR_NONFINITE, "adjoint: the loss is NaN or Inf");
    if (loss) *loss = A.loss;
    if (nforward_steps) *nforward_steps = A.fwd_steps;
    release();
    A.release_graphs();
    return st;
}

}  // extern "C"
