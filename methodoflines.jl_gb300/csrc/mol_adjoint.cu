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
// States between checkpoints are recomputed; checkpoint positions follow the
// binomial (revolve) schedule of Griewank & Walther for `nsnap` slots.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mol_kernels.cuh"
#include "mol_plan.h"

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

__global__ void k_set_t(SolverState* S, double t) {
    S->t = t;
    S->blocks_done = 0;
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
    double *work, *u1, *u2, *lam, *l2, *l1, *tmp;
    double* lam_p;
    double* lam_aux;
    bool have_lam = false;
    double loss = 0.0;
    double* uT_dev = nullptr;
    long long fwd_steps = 0;
    int err = MOL_OK;

    int ck(cudaError_t e, const char* w) {
        if (err) return err;
        err = cuda_check(plan, e, w);
        return err;
    }

    void set_time(double t) {
        k_set_t<<<1, 1, 0, plan->stream>>>(plan->d_state, t);
        ++g_launches;
    }

    // state at step `from` in src -> state at step `from + k` in dst
    void advance(const double* src, double* dst, int64_t from, int64_t k) {
        if (err) return;
        if (dst != src) ck(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, plan->stream), "copy");
        set_time(t0 + from * dt);
        for (int64_t s = 0; s < k && !err; ++s) {
            int st = launch_ssprk_step<double>(plan, dst, u1, u2, p, dt);
            if (st) err = st;
        }
        fwd_steps += k;
    }

    void vjp(const double* seed, double scale, const double* u, double t, double* out) {
        if (err) return;
        const DevProb<double>& P = plan->P64;
        const double* cseed = seed;
        cudaError_t e = launch_k(plan->jit.vjp64, plan->nblocks, plan->nthreads, plan->stream, P, cseed, scale, u, p, t,
                                 out, lam_p, lam_aux);
        ++g_launches;
        ck(e, "vjp launch");
    }

    void stage(int which, const double* uin, const double* u0, double* uout, double t) {
        if (err) return;
        const DevProb<double>& P = plan->P64;
        const double* cu = uin;
        cudaError_t e = launch_k(plan->jit.ssp64[which - 1], plan->nblocks, plan->nthreads, plan->stream, P, cu, u0, uout,
                                 p, plan->d_state, dt, t);
        ++g_launches;
        ck(e, "stage launch");
    }

    // Reverse step m, the state u_m being in `um`.
    void reverse_step(const double* um, int64_t m) {
        if (err) return;
        const double tm = t0 + m * dt;
        stage(1, um, um, u1, tm);
        stage(2, u1, um, u2, tm);
        fwd_steps += 1;
        if (!have_lam) {
            // last step: u_N and dL/du_N
            stage(3, u2, um, tmp, tm);
            if (uT_dev) ck(cudaMemcpyAsync(uT_dev, tmp, sizeof(double) * n, cudaMemcpyDeviceToDevice, plan->stream), "uT");
            if (loss_kind == MOL_LOSS_MISFIT) {
                k_misfit<<<nb, kThreads, 0, plan->stream>>>(n, tmp, target, lam, plan->d_partials);
                ++g_launches;
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
        // l2 = 2/3 lam + (2dt/3) J(u2)^T lam
        k_lincomb3<<<nb, kThreads, 0, plan->stream>>>(n, l2, 2.0 / 3.0, lam, 0.0, nullptr, 0.0, nullptr);
        vjp(lam, 2.0 * dt / 3.0, u2, tm + dt / 2, l2);
        // l1 = 1/4 l2 + (dt/4) J(u1)^T l2
        k_lincomb3<<<nb, kThreads, 0, plan->stream>>>(n, l1, 0.25, l2, 0.0, nullptr, 0.0, nullptr);
        vjp(l2, dt / 4.0, u1, tm + dt, l1);
        // lam = 1/3 lam + 3/4 l2 + l1 + dt J(u)^T l1
        k_lincomb3<<<nb, kThreads, 0, plan->stream>>>(n, lam, 1.0 / 3.0, lam, 0.75, l2, 1.0, l1);
        vjp(l1, dt, um, tm, lam);
        g_launches += 3;
    }

    static double beta(int s, int t) {  // C(s + t, t), saturating
        double b = 1.0;
        for (int i = 1; i <= t; ++i) {
            b = b * (s + i) / i;
            if (b > 1e18) return 1e18;
        }
        return b;
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
        const int s = (int)free.size();
        const int64_t nn = r - l;
        int t = 1;
        while (beta(s, t) < (double)nn) ++t;
        int64_t left = (int64_t)std::min<double>(beta(s, t - 1), (double)(nn - 1));
        left = std::max<int64_t>(1, left);
        const int64_t m = l + left;
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
    cudaError_t e = launch_k(plan->jit.vjp64, plan->nblocks, plan->nthreads, plan->stream, P, dl, 1.0, du, pp, t, ou,
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
    if (!plan || !u0 || !target || nsteps < 0 || !(dt > 0) || (loss_kind != MOL_LOSS_MISFIT && loss_kind != MOL_LOSS_LAMBDA))
        return MOL_ERR_INVALID;
    int st = need_vjp(plan);
    if (st) return st;
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
    // checkpoint slots: nsnap <= 0 stores every step that fits in half of the free memory
    int64_t slots = nsnap;
    if (slots <= 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        slots = (int64_t)std::max<double>(2.0, std::min<double>((double)nsteps + 1, 0.5 * fr / (8.0 * n)));
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
    for (int64_t i = 0; i < slots; ++i) {
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
    A.l2 = get(n);
    A.l1 = get(n);
    A.tmp = get(n);
    A.target = get(n);
    A.lam_p = get(std::max(plan->nparams, 1));
    A.lam_aux = get((size_t)std::max<long long>(plan->aux_total, 1));
    double* pbuf = get(std::max(plan->nparams, 1));
    if (!A.work || !A.u1 || !A.u2 || !A.lam || !A.l2 || !A.l1 || !A.tmp || !A.target || !A.lam_p || !A.lam_aux || !pbuf) {
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
        std::vector<double*> free(A.slots.begin() + 1, A.slots.end());
        A.rev(0, nsteps, A.slots[0], free);
    }
    st = A.err;
    if (!st && uT) st = dev_out(plan, uT, A.uT_dev, n);
    if (!st && dLdu0) st = dev_out(plan, dLdu0, A.lam, n);
    if (!st && dLdp && plan->nparams > 0) st = dev_out(plan, dLdp, A.lam_p, plan->nparams);
    if (!st && dLdaux && plan->aux_total > 0) st = dev_out(plan, dLdaux, A.lam_aux, plan->aux_total);
    if (!st) st = cuda_check(plan, cudaStreamSynchronize(plan->stream), "adjoint sync");
    if (loss) *loss = A.loss;
    if (nforward_steps) *nforward_steps = A.fwd_steps;
    release();
    return st;
}

}  // extern "C"
