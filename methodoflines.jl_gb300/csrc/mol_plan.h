// Host-side plan shared by the translation units of libmolgpu.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "mol_codegen.h"
#include "mol_device.cuh"
#include "molgpu.h"

namespace mol {

extern std::atomic<long long> g_launches;

struct PlanArrays {
    // per-precision copies of everything the kernels read
    void* w = nullptr;
    void* consts = nullptr;
    void* aux = nullptr;
    void* coords[3] = {nullptr, nullptr, nullptr};
    void* bc = nullptr;
    void* params = nullptr;
    // host copy of what `params` holds (valid when params_known), so a call passing the
    // same host parameters again skips the upload
    std::vector<double> params_host;
    bool params_known = false;
};

struct mol_plan_impl;

constexpr int kMaxSlabs = 8;  // slabs of the streamed host-to-device copy

}  // namespace mol

struct mol_plan {
    int dev = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    mol_problem_desc desc{};          // scalar fields only (pointers not retained)
    long long nunk = 0, ncell = 0;
    int nfields = 0, nparams = 0, naux = 0;
    long long aux_total = 0;
    std::vector<long long> aux_off_host;
    std::vector<double> params_host;
    // structure arrays (precision independent)
    mol_op1d* d_ops = nullptr;
    mol_term* d_terms = nullptr;
    mol_instr* d_code = nullptr;
    int* d_progs = nullptr;
    long long* d_aux_off = nullptr;
    mol::PlanArrays a64, a32;
    mol::DevProb<double> P64{};
    mol::DevProb<float> P32{};
    // workspaces
    std::vector<void*> allocs;
    double* ws64[12] = {nullptr};
    float* ws32[12] = {nullptr};
    mol::SolverState* d_state = nullptr;
    double* d_partials = nullptr;
    int nblocks = 0;
    int nblocks32 = 0, nthreads32 = 0;   // grid of the Float32-state kernels (own register budget)
    // grid of the face pass: it moves more bytes per FP64 operation than the stage kernels
    // and needs more warps in flight, so it runs at its own (higher) occupancy
    int face_blocks = 0, face_threads = 256;
    int vjp_blocks = 0;   // grid of the vector-Jacobian product (its own register budget)
    int sms = 152;
    int nthreads = 256;
    // adjoint workspaces
    double* adj[16] = {nullptr};
    double* d_snap = nullptr;
    long long nsnap_alloc = 0;
    double* d_lam_p_partials = nullptr;
    // cached CUDA graphs for fixed-step SSPRK33 chunks
    cudaGraphExec_t g_ssp64 = nullptr, g_ssp32 = nullptr;
    double g_ssp64_dt = 0, g_ssp32_dt = 0;
    const void* g_ssp64_p = nullptr;
    const void* g_ssp32_p = nullptr;
    const void* g_ssp64_pp = nullptr;
    const void* g_ssp32_pp = nullptr;
    int g_chunk = 16;
    // generated right-hand side (NVRTC); the interpreter serves when it is off
    mol::JitKernels jit;
    bool use_jit = false;
    std::string jit_src, jit_err;
    // face pass for nonlinear-Laplacian terms: nface slots of ncell left faces per precision
    int nface = 0;
    bool face_pass = false;
    double* faces64 = nullptr;
    float* faces32 = nullptr;
    // coefficient stencils: ncoef per-cell coefficient arrays (k_coef_t), FP64 and FP32
    int ncoef = 0;
    double* coef64 = nullptr;
    float* coef32 = nullptr;
    // device staging of full-grid output (mol_fill_grid) for host destinations
    double* grid_buf = nullptr;
    long long grid_cap = 0;
    // host-to-device copy of a pinned state in slabs of the slowest dimension, overlapped
    // with stage 1 (h2d_slabs < 2: one copy before the step)
    int h2d_slabs = 0;
    long long halo = 0;      // slices a stencil reaches along the slowest dimension
    bool per_last = false;   // the slowest dimension is periodic
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t slab_ev[mol::kMaxSlabs + 1] = {nullptr};
};

namespace mol {

int set_err(mol_plan* plan, int code, const std::string& msg);
int cuda_check(mol_plan* plan, cudaError_t e, const char* what);
bool is_device_ptr(const void* p);
int plan_alloc(mol_plan* plan, void** ptr, size_t bytes);
int plan_grid(const mol_plan* plan);
int grid_for(long long ncell, int sms, int blocks_per_sm);
int threads_for(long long ncell, int sms, int blocks_per_sm);
int plan_create_impl(const mol_problem_desc* d, mol_plan** out, bool member);
// Synchronises the plan's stream and returns MOL_ERR_NONFINITE (clearing the flag) when an
// SSPRK33 step since the last check produced a NaN or Inf state value.
int sync_and_check_finite(mol_plan* plan);

template <class T>
DevProb<T>& prob(mol_plan* plan);
template <>
inline DevProb<double>& prob<double>(mol_plan* plan) { return plan->P64; }
template <>
inline DevProb<float>& prob<float>(mol_plan* plan) { return plan->P32; }

template <class T>
T** workspace(mol_plan* plan);
template <>
inline double** workspace<double>(mol_plan* plan) { return plan->ws64; }
template <>
inline float** workspace<float>(mol_plan* plan) { return plan->ws32; }

template <class T>
int ensure_ws(mol_plan* plan, int count);

// launch helpers implemented in mol_plan.cu
template <class T>
int launch_rhs(mol_plan* plan, T* du, const T* u, const T* p, double t);
template <class T>
int launch_ssprk_step(mol_plan* plan, T* u, T* u1, T* u2, const T* p, double dt);
template <class T>
int launch_ssprk_step_io(mol_plan* plan, const T* uin, T* uout, T* u1, T* u2, const T* p, double dt,
                         bool skip1 = false);
void* mapped_host_ptr(const void* p);
// The face pass of nonlinear-Laplacian terms (see k_faces_t): buffer allocation (before any
// capture) and the launch, returning the problem view the next cell kernel takes.
template <class T>
int ensure_faces(mol_plan* plan);
template <class T>
DevProb<T> with_faces(mol_plan* plan, const T* u, const T* p, double toff, double tfix, cudaError_t* e);

}  // namespace mol
