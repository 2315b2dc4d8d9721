// Generated right-hand side (see mol_codegen.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "molgpu.h"

namespace mol {

enum { JIT_FWD64 = 0, JIT_FWD32 = 1, JIT_BATCH = 2, JIT_VJP = 3 };

// Kernels of a generated module; groups other than the FP64 forward kernels are
// compiled on first use.
struct JitKernels {
    bool ok = false;
    unsigned loaded = 0;
    std::string src;
    int nparams = 0;
    int min_blocks = 2;
    cudaKernel_t rhs64 = nullptr, ssp64[3] = {nullptr, nullptr, nullptr}, batch64 = nullptr, tsit64 = nullptr;
    cudaKernel_t rhs32 = nullptr, ssp32[3] = {nullptr, nullptr, nullptr}, batch32 = nullptr, tsit32 = nullptr;
    cudaKernel_t vjp64 = nullptr;
    cudaKernel_t tiles64 = nullptr, tiles32 = nullptr;
    cudaKernel_t faces64 = nullptr, faces32 = nullptr;  // face pass (nonlinear Laplacian)
};

std::string generate_source(const mol_problem_desc* d, std::string& why);
// True when the generated code evaluates nonlinear-Laplacian term k in its folded form: the
// outer and inner operators are two-point antisymmetric stencils (w[0] == -w[1], the
// second-order half-offset first derivative), so a face is stored as a * (u[I+1] - u[I])
// and the cell forms (wo[1] wi[1]) * (F'(I+1/2) - F'(I-1/2)).  The library then appends
// wo[1] * wi[1] and 1 / wi[1] to the weight pool at the term's reserved0 offset.
// MOL_JIT_FOLD=0 turns the folded form off.
bool nonlinlap_fold(const mol_problem_desc* d, int k);

// Constant-coefficient fusion of first-derivative stencils.  In the sum that forms one
// output of the cell program, the addends c * T with c a compile-time constant and T a
// first-derivative stencil of one field (a LINEAR term with antisymmetric interior weights,
// a MIXED term, or the stencil an UPWIND select picks for the constant's sign) are evaluated
// as one stencil over the union of their taps, with weights sum(c * w) precomputed per plan
// (appended to the weight pool; the offset is stored in terms[key_term].reserved2).  Second
// derivatives are left alone: folding a constant into a 1/dx^2 stencil changes the rounding
// of its cancelling sum by far more than the 1e-12 parity bar.  MOL_JIT_CFOLD=0 turns it off.
struct FoldPart {
    int term;      // member term
    int m;         // interior weight index (MIXED: x * L2 + y)
    double coef;   // the constant, sign included
};
struct FoldTap {
    int o[3];
    std::vector<FoldPart> parts;
};
struct FoldGroup {
    int out_pc = -1;                        // OUT instruction of the cell program
    int field = -1;
    int key_term = -1;
    std::vector<std::pair<double, int>> folded;   // (sign, leaf pc) in addend order
    std::vector<std::pair<double, int>> rest;     // the other addends, in order
    std::vector<int> absorbed;              // pcs emitted only on the fallback path (or not at all)
    std::vector<int> leaf_nodes;            // pcs of the folded leaves' subtrees (fallback path)
    std::vector<FoldTap> taps;
};
std::vector<FoldGroup> const_linear_groups(const mol_problem_desc* d);
// The fused weights of a group, one per tap (sum over its parts of coefficient * weight).
std::vector<double> fold_weights(const mol_problem_desc* d, const FoldGroup& g);
std::vector<std::string> jit_kernel_names(int nparams, int group);
// Generates, compiles (NVRTC, sm_103a) and loads the module of a problem structure;
// modules are cached per generated source for the life of the process.
int jit_compile(const mol_problem_desc* d, JitKernels* out, std::string& err, std::string* src_out, int min_blocks);
// NVRTC compile of generated source (no device needed); cubin and lowered kernel names optional.
int nvrtc_compile(const std::string& src, int nparams, int group, std::vector<char>* cubin,
                  std::vector<std::string>* lowered, std::string& err, int min_blocks = 2);
// Compiles and loads a kernel group of an already generated module on first use.
int jit_ensure(JitKernels* k, int group, std::string& err);

template <class... A>
cudaError_t launch_k(cudaKernel_t k, int grid, int block, cudaStream_t s, A... args) {
    void* pa[] = {(void*)&args...};
    return cudaLaunchKernel((const void*)k, dim3(grid), dim3(block), pa, 0, s);
}
// The same with `smem` bytes of dynamic shared memory per CTA.
template <class... A>
cudaError_t launch_ks(cudaKernel_t k, int grid, int block, size_t smem, cudaStream_t s, A... args) {
    void* pa[] = {(void*)&args...};
    return cudaLaunchKernel((const void*)k, dim3(grid), dim3(block), pa, smem, s);
}

}  // namespace mol
