// Batched ensemble: many instances of one PDE structure with uneven grids.
//
// Every instance is lowered on the host exactly like a single problem; the
// ensemble then runs one persistent kernel in which each CTA takes the next
// instance (largest first, handed out by an atomic ticket) and integrates it
// for all requested SSPRK33 steps, synchronising only its own threads between
// stages.  There is no grid-wide barrier and no inter-CTA wait.  The launch
// (ticket reset + kernel) is captured once in a CUDA graph and replayed.
// Threads per CTA and CTAs per SM are autotuned on the ensemble itself.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <numeric>
#include <string>
#include <vector>

#include "mol_kernels.cuh"
#include "mol_plan.h"

using namespace mol;

struct mol_batch {
    int dev = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    int n = 0;
    std::vector<mol_plan*> plans;
    std::vector<long long> off;   // packed offsets (n + 1)
    long long total = 0;
    long long max_cells = 0;
    JitKernels jit;
    std::string src;
    DevProb<double>* d_p64 = nullptr;
    DevProb<float>* d_p32 = nullptr;
    long long* d_off = nullptr;
    int* d_order = nullptr;
    double* d_dt = nullptr;
    unsigned* d_ticket = nullptr;
    const double** d_par64 = nullptr;
    const float** d_par32 = nullptr;
    double* s64[3] = {nullptr, nullptr, nullptr};  // state (staging), u1, u2
    float* s32[3] = {nullptr, nullptr, nullptr};
    int threads = 256, ctas_per_sm = 2, sms = 152;
    bool tuned = false;
    std::vector<void*> allocs;
    cudaGraphExec_t graph = nullptr;
    const void* g_key[4] = {nullptr, nullptr, nullptr, nullptr};
    long long g_steps = -1;
    double g_t0 = 0.0;
    int g_cfg[2] = {0, 0};
};

namespace {

int berr(mol_batch* b, int code, const std::string& m) {
    if (b) b->err = m;
    return code;
}

int bcheck(mol_batch* b, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return MOL_OK;
    cudaGetLastError();
    return berr(b, e == cudaErrorMemoryAllocation ? MOL_ERR_OOM : MOL_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

int balloc(mol_batch* b, void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return bcheck(b, e, "cudaMalloc");
    b->allocs.push_back(*p);
    return MOL_OK;
}

template <class T>
int run(mol_batch* b, T* U, const double* dts_host, double t0, long long nsteps, int threads, int ctas) {
    const bool is64 = std::is_same<T, double>::value;
    T* const* S = nullptr;
    (void)S;
    T* U1 = is64 ? (T*)b->s64[1] : (T*)b->s32[1];
    T* U2 = is64 ? (T*)b->s64[2] : (T*)b->s32[2];
    const DevProb<T>* probs = is64 ? (const DevProb<T>*)b->d_p64 : (const DevProb<T>*)b->d_p32;
    const T* const* params = is64 ? (const T* const*)b->d_par64 : (const T* const*)b->d_par32;
    cudaKernel_t k = is64 ? b->jit.batch64 : b->jit.batch32;
    int st;
    if (dts_host)
        if ((st = bcheck(b, cudaMemcpyAsync(b->d_dt, dts_host, sizeof(double) * b->n,
                                            is_device_ptr(dts_host) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                            b->stream), "dt")))
            return st;
    const int grid = b->sms * ctas;
    const long long* off = b->d_off;
    const int* order = b->d_order;
    const int ninst = b->n;
    unsigned* ticket = b->d_ticket;
    // one replayable graph: ticket reset + persistent kernel
    const bool key_ok = b->graph && b->g_key[0] == (const void*)U && b->g_key[1] == (const void*)k &&
                        b->g_steps == nsteps && b->g_t0 == t0 && b->g_cfg[0] == threads && b->g_cfg[1] == ctas;
    const bool can_capture = b->stream != nullptr && b->stream != cudaStreamLegacy;
    if (!key_ok && can_capture) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        cudaGraph_t g;
        if ((st = bcheck(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "capture"))) return st;
        cudaMemsetAsync(ticket, 0, sizeof(unsigned), b->stream);
        launch_k(k, grid, threads, b->stream, probs, off, order, ninst, U, U1, U2, params, (const double*)b->d_dt, t0,
                 nsteps, ticket);
        if ((st = bcheck(b, cudaStreamEndCapture(b->stream, &g), "end capture"))) return st;
        st = bcheck(b, cudaGraphInstantiate(&b->graph, g, 0), "instantiate");
        cudaGraphDestroy(g);
        if (st) return st;
        b->g_key[0] = U;
        b->g_key[1] = k;
        b->g_steps = nsteps;
        b->g_t0 = t0;
        b->g_cfg[0] = threads;
        b->g_cfg[1] = ctas;
    }
    ++g_launches;
    if (can_capture) return bcheck(b, cudaGraphLaunch(b->graph, b->stream), "batch graph launch");
    cudaMemsetAsync(ticket, 0, sizeof(unsigned), b->stream);
    return bcheck(b, launch_k(k, grid, threads, b->stream, probs, off, order, ninst, U, U1, U2, params,
                              (const double*)b->d_dt, t0, nsteps, ticket), "batch launch");
}

template <class T>
int tune(mol_batch* b, T* U, long long probe_steps) {
    // Candidates within the register budget of the kernel (launch bound 256 threads).
    cudaFuncAttributes fa;
    int regs = 128;
    if (cudaFuncGetAttributes(&fa, (const void*)(std::is_same<T, double>::value ? b->jit.batch64 : b->jit.batch32)) ==
            cudaSuccess && fa.numRegs > 0)
        regs = fa.numRegs;
    else
        cudaGetLastError();
    std::vector<std::pair<int, int>> cand;
    for (int th : {128, 256})
        for (int c : {1, 2, 3, 4, 6, 8})
            if ((long long)th * c * regs <= 65536 && th * c <= 2048) cand.push_back({th, c});
    if (cand.empty()) cand.push_back({128, 1});
    // time on a scratch copy of the state so tuning leaves the caller's data alone
    T* scratch = nullptr;
    if (cudaMalloc(&scratch, sizeof(T) * b->total) != cudaSuccess) {
        cudaGetLastError();
        return MOL_OK;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    std::pair<int, int> pick = cand[0];
    for (auto& c : cand) {
        cudaMemcpyAsync(scratch, U, sizeof(T) * b->total, cudaMemcpyDeviceToDevice, b->stream);
        cudaEventRecord(e0, b->stream);
        int st = run<T>(b, scratch, nullptr, 0.0, probe_steps, c.first, c.second);
        cudaEventRecord(e1, b->stream);
        cudaEventSynchronize(e1);
        if (st) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            pick = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(scratch);
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    b->threads = pick.first;
    b->ctas_per_sm = pick.second;
    b->tuned = true;
    return MOL_OK;
}

template <class T>
int step_impl(mol_batch* b, T* u, const double* dts, double t0, int64_t nsteps) {
    if (!b || !u || !dts || nsteps < 0) return MOL_ERR_INVALID;
    int st;
    const bool is64 = std::is_same<T, double>::value;
    if ((st = jit_ensure(&b->jit, JIT_BATCH, b->err))) return berr(b, st, b->err);
    T** S = is64 ? (T**)b->s64 : (T**)b->s32;
    for (int i = 0; i < 3; ++i)
        if (!S[i] && (st = balloc(b, (void**)&S[i], sizeof(T) * b->total))) return st;
    const bool host = !is_device_ptr(u);
    T* U = host ? S[0] : u;
    if (host && (st = bcheck(b, cudaMemcpyAsync(U, u, sizeof(T) * b->total, cudaMemcpyHostToDevice, b->stream), "H2D")))
        return st;
    if ((st = bcheck(b, cudaMemcpyAsync(b->d_dt, dts, sizeof(double) * b->n,
                                        is_device_ptr(dts) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                        b->stream), "dt")))
        return st;
    if (!b->tuned && nsteps > 0) tune<T>(b, U, std::min<int64_t>(nsteps, 2));
    if ((st = run<T>(b, U, nullptr, t0, nsteps, b->threads, b->ctas_per_sm))) return st;
    if (host) {
        if ((st = bcheck(b, cudaMemcpyAsync(u, U, sizeof(T) * b->total, cudaMemcpyDeviceToHost, b->stream), "D2H")))
            return st;
        return bcheck(b, cudaStreamSynchronize(b->stream), "sync");
    }
    return bcheck(b, cudaGetLastError(), "batch");
}

}  // namespace

extern "C" {

int mol_batch_create(const mol_problem_desc* const* descs, int32_t n, mol_batch** out) {
    if (!out) return MOL_ERR_INVALID;
    *out = nullptr;
    if (!descs || n < 1) return MOL_ERR_INVALID;
    mol_batch* b = new mol_batch();
    *out = b;
    cudaGetDevice(&b->dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->dev);
    b->n = n;
    int st;
    // every member must generate the same code: one structure, one module
    std::string why;
    b->src = generate_source(descs[0], why);
    if (b->src.empty()) return berr(b, MOL_ERR_UNSUPPORTED, "codegen: " + why);
    b->off.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        mol_plan* p = nullptr;
        st = plan_create_impl(descs[i], &p, true);
        if (st) {
            std::string m = p ? p->err : "plan creation failed";
            if (p) mol_plan_destroy(p);
            return berr(b, st, "instance " + std::to_string(i) + ": " + m);
        }
        b->plans.push_back(p);
        if (i > 0 && (descs[i]->nparams != descs[0]->nparams || descs[i]->nfields != descs[0]->nfields)) {
            return berr(b, MOL_ERR_INVALID, "instance " + std::to_string(i) + " differs in structure");
        }
        b->off[i + 1] = b->off[i] + p->nunk;
        b->max_cells = std::max(b->max_cells, p->ncell);
    }
    // spot-check structure identity (first, last and a stride of members)
    for (int i = 1; i < n; i += std::max(1, n / 16)) {
        if (generate_source(descs[i], why) != b->src)
            return berr(b, MOL_ERR_INVALID, "instance " + std::to_string(i) + " has a different term structure");
    }
    b->total = b->off[n];
    std::string err;
    b->jit.src = b->src;
    b->jit.nparams = descs[0]->nparams;
    b->jit.ok = true;
    if ((st = jit_ensure(&b->jit, JIT_BATCH, err))) return berr(b, st, err);
    if ((st = bcheck(b, cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream"))) return st;
    b->own_stream = true;
    std::vector<DevProb<double>> p64(n);
    std::vector<DevProb<float>> p32(n);
    std::vector<const double*> par64(n);
    std::vector<const float*> par32(n);
    for (int i = 0; i < n; ++i) {
        p64[i] = b->plans[i]->P64;
        p32[i] = b->plans[i]->P32;
        par64[i] = (const double*)b->plans[i]->a64.params;
        par32[i] = (const float*)b->plans[i]->a32.params;
    }
    // largest instances first (longest-processing-time order for the dynamic ticket)
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int c) { return b->plans[a]->ncell > b->plans[c]->ncell; });
    if ((st = balloc(b, (void**)&b->d_p64, sizeof(DevProb<double>) * n))) return st;
    if ((st = balloc(b, (void**)&b->d_p32, sizeof(DevProb<float>) * n))) return st;
    if ((st = balloc(b, (void**)&b->d_off, sizeof(long long) * (n + 1)))) return st;
    if ((st = balloc(b, (void**)&b->d_order, sizeof(int) * n))) return st;
    if ((st = balloc(b, (void**)&b->d_dt, sizeof(double) * n))) return st;
    if ((st = balloc(b, (void**)&b->d_ticket, sizeof(unsigned)))) return st;
    if ((st = balloc(b, (void**)&b->d_par64, sizeof(void*) * n))) return st;
    if ((st = balloc(b, (void**)&b->d_par32, sizeof(void*) * n))) return st;
    cudaMemcpy(b->d_p64, p64.data(), sizeof(DevProb<double>) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(b->d_p32, p32.data(), sizeof(DevProb<float>) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(b->d_off, b->off.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(b->d_order, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
    cudaMemcpy(b->d_par64, par64.data(), sizeof(void*) * n, cudaMemcpyHostToDevice);
    st = bcheck(b, cudaMemcpy(b->d_par32, par32.data(), sizeof(void*) * n, cudaMemcpyHostToDevice), "upload");
    return st;
}

int mol_batch_destroy(mol_batch* b) {
    if (!b) return MOL_ERR_INVALID;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->graph) cudaGraphExecDestroy(b->graph);
    for (mol_plan* p : b->plans) mol_plan_destroy(p);
    for (void* p : b->allocs) cudaFree(p);
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return MOL_OK;
}

const char* mol_batch_last_error(const mol_batch* b) { return b ? b->err.c_str() : "null batch"; }

int mol_batch_set_stream(mol_batch* b, void* stream) {
    if (!b) return MOL_ERR_INVALID;
    if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
    b->own_stream = false;
    b->stream = (cudaStream_t)stream;
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return MOL_OK;
}

int mol_batch_offsets(const mol_batch* b, int64_t* offsets) {
    if (!b || !offsets) return MOL_ERR_INVALID;
    for (int i = 0; i <= b->n; ++i) offsets[i] = b->off[i];
    return MOL_OK;
}

int mol_batch_step_ssprk33(mol_batch* b, double* u, const double* dts, double t0, int64_t nsteps) {
    return step_impl<double>(b, u, dts, t0, nsteps);
}

int mol_batch_step_ssprk33_f32state(mol_batch* b, float* u, const double* dts, double t0, int64_t nsteps) {
    return step_impl<float>(b, u, dts, t0, nsteps);
}

int mol_batch_tune(mol_batch* b, int32_t threads, int32_t ctas_per_sm, int64_t smem_cells) {
    if (!b) return MOL_ERR_INVALID;
    (void)smem_cells;
    if (threads > 0) {
        if (threads % 32 || threads > 256) return berr(b, MOL_ERR_INVALID, "threads must be a multiple of 32, <= 256");
        b->threads = threads;
        b->tuned = true;
    }
    if (ctas_per_sm > 0) {
        b->ctas_per_sm = ctas_per_sm;
        b->tuned = true;
    }
    if (threads == 0 && ctas_per_sm == 0) b->tuned = false;  // autotune again on the next run
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return MOL_OK;
}

}  // extern "C"
