// Batched ensemble: many instances of one PDE structure with uneven grids.
//
// Every instance is lowered on the host exactly like a single problem; the
// ensemble then runs one persistent kernel, captured once in a CUDA graph with
// the resets of its work counters and replayed.  Two schedules:
//  - tiles (default): the work unit is one tile of one SSPRK33 stage of one
//    instance; a 64-bit ticket hands units out round by round (largest instances
//    first) and a per-instance counter of finished tiles orders the stages of an
//    instance across CTAs, so one large member spreads over the whole GPU;
//  - instances: each CTA takes the next whole instance and integrates it for all
//    steps, synchronising only its own threads between stages.
// Schedule, threads per CTA, CTAs per SM and tile size are autotuned on the
// ensemble itself.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
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
    // tiled schedule: [ticket u64][status i32 + pad][done u64 x n] in one allocation
    unsigned long long* d_sync = nullptr;
    TileRef* d_tiles = nullptr;              // per tile of a round: instance, index, count
    size_t d_tiles_cap = 0;
    int tile_cells_uploaded = 0;
    long long tiles_total = 0;               // tiles of one round at the uploaded tile size
    unsigned long long inject_ticket = 0;     // host value for the injected first ticket
    const double** d_par64 = nullptr;
    const float** d_par32 = nullptr;
    double* s64[3] = {nullptr, nullptr, nullptr};  // state (staging), u1, u2
    float* s32[3] = {nullptr, nullptr, nullptr};
    int threads = 256, ctas_per_sm = 2, sms = 152;
    int tile_cells = 2048;   // > 0 tiled schedule, 0 one CTA per instance
    int nface = 0;           // nonlinear-Laplacian terms (faces shared through shared memory)
    bool tuned = false;
    std::vector<void*> allocs;
    cudaGraphExec_t graph = nullptr;
    const void* g_key[4] = {nullptr, nullptr, nullptr, nullptr};
    long long g_steps = -1;
    double g_t0 = 0.0;
    int g_cfg[3] = {0, 0, 0};
    std::vector<int> order;       // slot -> instance (largest first)
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

// Shared-memory face window of the tiled kernel for state type T: bytes per CTA (0: off) and
// cells per face term.  MOL_BATCH_FACE_BYTES sets the bytes (0 turns the window off).
template <class T>
void face_window(const mol_batch* b, size_t* bytes, long long* cells) {
    *bytes = 0;
    *cells = 0;
    // FP64 state only: the Float32-state ensemble is not bound by its face arithmetic, and the
    // window's barriers made it slower (1000 steps of the 4096 members: 25.5 s -> 33.5 s)
    if (b->nface <= 0 || sizeof(T) != sizeof(double)) return;
    long long want = 45056;
    if (const char* e = getenv("MOL_BATCH_FACE_BYTES")) want = std::max(0ll, std::min(atoll(e), 48ll * 1024));
    const long long w = want / ((long long)b->nface * (long long)sizeof(T));
    if (w < 64) return;
    *cells = w;
    *bytes = (size_t)w * b->nface * sizeof(T);
}

// The tile table of one round for a tile size: tiles of the instances in slot order
// (largest first), each with its instance, its index within the instance and the instance's
// tile count.
int upload_tiles(mol_batch* b, int tile_cells) {
    if (b->tile_cells_uploaded == tile_cells) return MOL_OK;
    std::vector<TileRef> t;
    for (int s = 0; s < b->n; ++s) {
        const int inst = b->order[s];
        const long long nc = b->plans[inst]->ncell;
        const long long k = (nc + tile_cells - 1) / tile_cells;
        for (long long j = 0; j < k; ++j) t.push_back(TileRef{inst, (int)j, (int)k, 0});
    }
    int st = MOL_OK;
    if (t.size() > b->d_tiles_cap) {
        if (b->d_tiles) cudaFree(b->d_tiles);
        b->d_tiles = nullptr;
        b->d_tiles_cap = 0;
        void* q = nullptr;
        if ((st = bcheck(b, cudaMalloc(&q, sizeof(TileRef) * t.size()), "tile table"))) return st;
        b->d_tiles = (TileRef*)q;
        b->d_tiles_cap = t.size();
    }
    st = bcheck(b, cudaMemcpyAsync(b->d_tiles, t.data(), sizeof(TileRef) * t.size(), cudaMemcpyHostToDevice,
                                   b->stream), "tile table");
    if (!st) st = bcheck(b, cudaStreamSynchronize(b->stream), "tile table");
    if (!st) {
        b->tile_cells_uploaded = tile_cells;
        b->tiles_total = (long long)t.size();
    }
    return st;
}

template <class T>
int run(mol_batch* b, T* U, double t0, long long nsteps, int threads, int ctas, int tile_cells) {
    const bool is64 = std::is_same<T, double>::value;
    T* U1 = is64 ? (T*)b->s64[1] : (T*)b->s32[1];
    T* U2 = is64 ? (T*)b->s64[2] : (T*)b->s32[2];
    const DevProb<T>* probs = is64 ? (const DevProb<T>*)b->d_p64 : (const DevProb<T>*)b->d_p32;
    const T* const* params = is64 ? (const T* const*)b->d_par64 : (const T* const*)b->d_par32;
    const bool tiled = tile_cells > 0;
    cudaKernel_t k = tiled ? (is64 ? b->jit.tiles64 : b->jit.tiles32) : (is64 ? b->jit.batch64 : b->jit.batch32);
    int st;
    if (tiled && (st = upload_tiles(b, tile_cells))) return st;
    const int grid = b->sms * ctas;
    const long long* off = b->d_off;
    const int* order = b->d_order;
    const int ninst = b->n;
    unsigned* ticket = b->d_ticket;
    BatchSync sync;
    sync.ticket = b->d_sync;
    sync.status = (int*)(b->d_sync + 1);
    sync.nonfinite = (int*)(b->d_sync + 1) + 1;
    sync.done = b->d_sync + 2;
    sync.spin_limit = MOL_BATCH_SPIN_LIMIT;
    // Host-side injection of a dependency that is never met, for tests of the bounded waits:
    // MOL_BATCH_INJECT_SKIP_ROUND=1 starts the ticket after round 0, so every tile of round 1
    // waits for round-0 tiles that no CTA will run; MOL_BATCH_SPIN_LIMIT shortens the budget.
    unsigned long long first_ticket = 0;
    if (const char* lim = getenv("MOL_BATCH_SPIN_LIMIT"))
        if (atoll(lim) > 0) sync.spin_limit = atoll(lim);
    if (tiled && getenv("MOL_BATCH_INJECT_SKIP_ROUND") && getenv("MOL_BATCH_INJECT_SKIP_ROUND")[0] == '1')
        first_ticket = (unsigned long long)b->tiles_total;
    const size_t sync_bytes = sizeof(unsigned long long) * (2 + (size_t)b->n);
    size_t fbytes = 0;
    long long fcells = 0;
    if (tiled) face_window<T>(b, &fbytes, &fcells);
    auto enqueue = [&]() -> cudaError_t {
        if (tiled) {
            // the status word survives replays so a failed run stays visible to mol_batch_check
            cudaError_t e = first_ticket ? cudaMemcpyAsync(b->d_sync, &b->inject_ticket, sizeof(unsigned long long),
                                                           cudaMemcpyHostToDevice, b->stream)
                                         : cudaMemsetAsync(b->d_sync, 0, sizeof(unsigned long long), b->stream);
            if (e == cudaSuccess)
                e = cudaMemsetAsync(b->d_sync + 2, 0, sync_bytes - 2 * sizeof(unsigned long long), b->stream);
            if (e != cudaSuccess) return e;
            return launch_ks(k, grid, threads, fbytes, b->stream, probs, off, (const TileRef*)b->d_tiles,
                             b->tiles_total, tile_cells, U, U1, U2, params, (const double*)b->d_dt, t0, nsteps, sync,
                             fcells);
        }
        cudaError_t e = cudaMemsetAsync(ticket, 0, sizeof(unsigned), b->stream);
        if (e != cudaSuccess) return e;
        return launch_k(k, grid, threads, b->stream, probs, off, order, ninst, U, U1, U2, params,
                        (const double*)b->d_dt, t0, nsteps, ticket, sync.nonfinite);
    };
    // one replayable graph: counter resets + persistent kernel
    const bool key_ok = b->graph && b->g_key[0] == (const void*)U && b->g_key[1] == (const void*)k &&
                        b->g_steps == nsteps && b->g_t0 == t0 && b->g_cfg[0] == threads && b->g_cfg[1] == ctas &&
                        b->g_cfg[2] == tile_cells;
    b->inject_ticket = first_ticket;
    const bool can_capture = b->stream != nullptr && b->stream != cudaStreamLegacy && !first_ticket &&
                             sync.spin_limit == MOL_BATCH_SPIN_LIMIT;
    if (!key_ok && can_capture) {
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        cudaGraph_t g;
        if ((st = bcheck(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "capture"))) return st;
        cudaError_t ee = enqueue();
        cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
        if ((st = bcheck(b, ee, "batch capture"))) return st;
        if ((st = bcheck(b, ec, "end capture"))) return st;
        st = bcheck(b, cudaGraphInstantiate(&b->graph, g, 0), "instantiate");
        cudaGraphDestroy(g);
        if (st) return st;
        b->g_key[0] = U;
        b->g_key[1] = k;
        b->g_steps = nsteps;
        b->g_t0 = t0;
        b->g_cfg[0] = threads;
        b->g_cfg[1] = ctas;
        b->g_cfg[2] = tile_cells;
    }
    ++g_launches;
    if (can_capture) return bcheck(b, cudaGraphLaunch(b->graph, b->stream), "batch graph launch");
    return bcheck(b, enqueue(), "batch launch");
}

// CTAs of `k` that fit on one SM at `threads` per CTA (0 if the query fails).
int resident_ctas(cudaKernel_t k, int threads, size_t smem = 0) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)k, threads, smem) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nb;
}

template <class T>
int tune(mol_batch* b, T* U, long long probe_steps) {
    const bool is64 = std::is_same<T, double>::value;
    struct Cand {
        int threads, ctas, tile;
    };
    std::vector<Cand> cand;
    for (int tiled = 0; tiled < 2; ++tiled) {
        cudaKernel_t k = tiled ? (is64 ? b->jit.tiles64 : b->jit.tiles32) : (is64 ? b->jit.batch64 : b->jit.batch32);
        size_t fbytes = 0;
        long long fcells = 0;
        if (tiled) face_window<T>(b, &fbytes, &fcells);
        for (int th : {128, 256}) {
            const int maxc = resident_ctas(k, th, fbytes);
            for (int c : {1, 2, 3, 4, 6, 8}) {
                if (c > maxc) continue;
                if (!tiled) cand.push_back({th, c, 0});
                else
                    for (int per : {4, 16, 64, 256}) cand.push_back({th, c, th * per});
            }
        }
    }
    if (cand.empty()) cand.push_back({128, 1, 0});
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
    Cand pick = cand[0];
    for (auto& c : cand) {
        cudaMemcpyAsync(scratch, U, sizeof(T) * b->total, cudaMemcpyDeviceToDevice, b->stream);
        cudaEventRecord(e0, b->stream);
        int st = run<T>(b, scratch, 0.0, probe_steps, c.threads, c.ctas, c.tile);
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
    b->threads = pick.threads;
    b->ctas_per_sm = pick.ctas;
    b->tile_cells = pick.tile;
    b->tuned = true;
    return MOL_OK;
}

template <class T>
int step_impl(mol_batch* b, T* u, const double* dts, double t0, int64_t nsteps) {
    if (!b || !u || !dts || nsteps < 0 || !std::isfinite(t0)) return MOL_ERR_INVALID;
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
    if ((st = run<T>(b, U, t0, nsteps, b->threads, b->ctas_per_sm, b->tile_cells))) return st;
    if (host) {
        if ((st = bcheck(b, cudaMemcpyAsync(u, U, sizeof(T) * b->total, cudaMemcpyDeviceToHost, b->stream), "D2H")))
            return st;
        return mol_batch_check(b);
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
    for (int k = 0; k < descs[0]->nterms; ++k)
        if (descs[0]->terms[k].kind == MOL_TERM_NONLINLAP) ++b->nface;
    b->off.assign(n + 1, 0);
    std::vector<int> cfold_shape;
    for (int i = 0; i < n; ++i) {
        mol_plan* p = nullptr;
        st = plan_create_impl(descs[i], &p, true);
        if (st) {
            std::string m = p ? p->err : "plan creation failed";
            if (p) mol_plan_destroy(p);
            return berr(b, st, "instance " + std::to_string(i) + ": " + m);
        }
        b->plans.push_back(p);
        if (i > 0 && (descs[i]->nparams != descs[0]->nparams || descs[i]->nfields != descs[0]->nfields ||
                      descs[i]->nterms != descs[0]->nterms)) {
            return berr(b, MOL_ERR_INVALID, "instance " + std::to_string(i) + " differs in structure");
        }
        // the shared module folds a nonlinear-Laplacian term only if every member's weights allow it
        for (int k = 0; i > 0 && k < descs[0]->nterms; ++k)
            if (nonlinlap_fold(descs[i], k) != nonlinlap_fold(descs[0], k))
                return berr(b, MOL_ERR_INVALID, "instance " + std::to_string(i) + " differs in structure (term " +
                                                    std::to_string(k) + " weights)");
        // and fuses the same constant-coefficient stencils (same taps) in every member
        if (i == 0) {
            for (const FoldGroup& g : const_linear_groups(descs[0])) cfold_shape.push_back((int)g.taps.size());
        } else {
            std::vector<int> shp;
            for (const FoldGroup& g : const_linear_groups(descs[i])) shp.push_back((int)g.taps.size());
            if (shp != cfold_shape)
                return berr(b, MOL_ERR_INVALID, "instance " + std::to_string(i) + " differs in structure (fused stencils)");
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
    b->jit.min_blocks = 2;
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
    b->order = order;
    if ((st = balloc(b, (void**)&b->d_sync, sizeof(unsigned long long) * (2 + (size_t)n)))) return st;
    cudaMemset(b->d_sync, 0, sizeof(unsigned long long) * (2 + (size_t)n));
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
    if (b->d_tiles) cudaFree(b->d_tiles);
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

int mol_batch_config(const mol_batch* b, int32_t* threads, int32_t* ctas_per_sm, int64_t* tile_cells) {
    if (!b) return MOL_ERR_INVALID;
    if (threads) *threads = b->threads;
    if (ctas_per_sm) *ctas_per_sm = b->ctas_per_sm;
    if (tile_cells) *tile_cells = b->tile_cells > 0 ? b->tile_cells : -1;
    return MOL_OK;
}

int mol_batch_check(mol_batch* b) {
    if (!b) return MOL_ERR_INVALID;
    int st = bcheck(b, cudaStreamSynchronize(b->stream), "batch sync");
    if (st) return st;
    int words[2] = {0, 0};  // status, nonfinite
    if ((st = bcheck(b, cudaMemcpy(words, (int*)(b->d_sync + 1), sizeof(words), cudaMemcpyDeviceToHost), "status")))
        return st;
    if (words[0] || words[1]) cudaMemset((int*)(b->d_sync + 1), 0, sizeof(words));
    if (words[0])
        return berr(b, MOL_ERR_CUDA, "batch: a stage dependency wait ran out of its poll budget; the run was abandoned");
    if (words[1])
        return berr(b, MOL_ERR_NONFINITE, "batch: a step produced a NaN or Inf state value (unstable)");
    return MOL_OK;
}

int mol_batch_tune(mol_batch* b, int32_t threads, int32_t ctas_per_sm, int64_t tile_cells) {
    if (!b) return MOL_ERR_INVALID;
    if (tile_cells != 0) {
        if (tile_cells > (1ll << 30)) return berr(b, MOL_ERR_INVALID, "tile_cells too large");
        b->tile_cells = tile_cells < 0 ? 0 : (int)tile_cells;
        b->tuned = true;
    }
    if (threads > 0) {
        if (threads % 32 || threads > 256) return berr(b, MOL_ERR_INVALID, "threads must be a multiple of 32, <= 256");
        b->threads = threads;
        b->tuned = true;
    }
    if (ctas_per_sm > 0) {
        b->ctas_per_sm = ctas_per_sm;
        b->tuned = true;
    }
    if (threads == 0 && ctas_per_sm == 0 && tile_cells == 0) b->tuned = false;  // autotune again on the next run
    if (b->graph) {
        cudaGraphExecDestroy(b->graph);
        b->graph = nullptr;
    }
    return MOL_OK;
}

}  // extern "C"
