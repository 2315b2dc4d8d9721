// Fixed-step SSPRK33 that allocates nothing.
//
// mol_step_ssprk33 keeps its two stage buffers (u1, u2) in the plan and allocates
// them on first use; it may also stage host arrays and instantiate a CUDA graph.
// Some callers cannot let a call allocate device memory: solver loops whose device
// memory budget is fixed up front (memory pools that must not grow, several plans
// sharing one GPU whose memory was divided between them at start-up), and host
// callbacks in which CUDA allocation calls are not allowed.  For them this variant
// takes its stage buffers from one file-scope device array instead.
//
// Limits and sharing:
//  - the array holds the stage buffers of at most MOL_NOALLOC_MAX_UNKNOWNS unknowns
//    (2 x 2^20 doubles = 16 MiB); every GPU that loads this library holds it until
//    the process exits;
//  - every call on a device uses the same array, so calls that overlap on the GPU
//    (different streams, or different plans on one stream without ordering) race;
//  - both stage buffers are written in full before they are read within a step, so
//    nothing in the array has to start at zero and stale contents of an earlier call
//    are never observed;
//  - the state `u` and parameters `p` must already be device memory; host arrays are
//    rejected because staging them would need a device buffer;
//  - the plan's generated FP64 kernels are compiled and loaded by mol_plan_create, so a
//    call loads no module; a nonlinear-Laplacian face buffer is used only if an earlier
//    mol_step_ssprk33 / mol_rhs call on the plan already made one (the kernels evaluate
//    the faces in the cell otherwise, with bit-identical results).
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "mol_kernels.cuh"
#include "mol_plan.h"

#define MOL_NOALLOC_MAX_UNKNOWNS (1ll << 20)

// Stage buffers u1 and u2, one after the other.
static __device__ __align__(256) double g_noalloc_scratch[2 * MOL_NOALLOC_MAX_UNKNOWNS];

namespace {

__global__ void k_noalloc_set_time(mol::SolverState* S, double t) {
    S->t = t;
    S->blocks_done = 0;
}

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on `dev` (which must be current).  In host code the
// array's name is only a host-side stand-in, so the address is looked up once per device.
int scratch_address(mol_plan* plan, int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) return mol::set_err(plan, MOL_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return mol::set_err(plan, MOL_ERR_CUDA,
                                std::string("cudaGetSymbolAddress(noalloc scratch): ") + cudaGetErrorString(e));
        }
        g_noalloc_ptr[dev] = (double*)p;
    }
    *out = g_noalloc_ptr[dev];
    return MOL_OK;
}

}  // namespace

extern "C" {

int mol_step_ssprk33_noalloc(mol_plan* plan, double* u, const double* p, double t0, double dt, int64_t nsteps) {
    if (!plan || !u || nsteps < 0) return MOL_ERR_INVALID;
    if (!std::isfinite(dt) || !std::isfinite(t0))
        return mol::set_err(plan, MOL_ERR_INVALID, "mol_step_ssprk33_noalloc: t0 and dt must be finite");
    if (plan->nunk > MOL_NOALLOC_MAX_UNKNOWNS)
        return mol::set_err(plan, MOL_ERR_INVALID,
                            "mol_step_ssprk33_noalloc: " + std::to_string(plan->nunk) +
                                " unknowns exceed the scratch limit of " + std::to_string(MOL_NOALLOC_MAX_UNKNOWNS));
    if (!mol::is_device_ptr(u))
        return mol::set_err(plan, MOL_ERR_INVALID, "mol_step_ssprk33_noalloc: u must be device memory");
    if (p && !mol::is_device_ptr(p))
        return mol::set_err(plan, MOL_ERR_INVALID, "mol_step_ssprk33_noalloc: p must be device memory or NULL");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != plan->dev) cudaSetDevice(plan->dev);
    double* scratch = nullptr;
    int st = scratch_address(plan, plan->dev, &scratch);
    // the FP64 group is loaded at plan creation; this only confirms it (no module load here)
    if (!st && plan->use_jit && !(plan->jit.loaded & (1u << mol::JIT_FWD64)))
        st = mol::set_err(plan, MOL_ERR_CUDA, "mol_step_ssprk33_noalloc: the plan's generated kernels are not loaded");
    if (!st) {
        const double* pp = p ? p : (const double*)plan->a64.params;
        double* u1 = scratch;
        double* u2 = scratch + MOL_NOALLOC_MAX_UNKNOWNS;
        k_noalloc_set_time<<<1, 1, 0, plan->stream>>>(plan->d_state, t0);
        ++mol::g_launches;
        for (int64_t s = 0; s < nsteps && !st; ++s) st = mol::launch_ssprk_step<double>(plan, u, u1, u2, pp, dt);
        if (!st) st = mol::cuda_check(plan, cudaGetLastError(), "mol_step_ssprk33_noalloc");
    }
    if (prev >= 0 && prev != plan->dev) cudaSetDevice(prev);
    return st;
}

}  // extern "C"
