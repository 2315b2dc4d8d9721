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
    cudaKernel_t coef64 = nullptr;                      // coefficient stencils (k_coef_t)
    cudaKernel_t tsitsmall64 = nullptr;                 // one-CTA Tsit5 for small problems
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
//
// Coefficient stencils.  A nonlinear-Laplacian addend Dj(a(x) Dj u) whose face coefficient
// depends on the coordinates only (its face program reads aux arrays and constants: a
// diffusivity field K(x)) and whose folded form applies joins the group as a *variable*
// member: its two faces contribute W a(I -/+ 1/2) (W = wo[1] wi[1]) to the taps of their
// inner differences.  Taps with a variable part read a per-cell coefficient array that
// k_coef_t fills once at plan creation (DevProb::cw, [array][cell]); the other taps keep
// their uniform weights.  Two evaluation forms:
//  - difference (default): every tap off the centre with a variable part is applied to
//    (u[tap] - u[centre]); the variable parts of the centre then cancel identically, so the
//    centre keeps only the constant parts (its own plus those of the differenced taps).  The
//    faces' arithmetic is the reference's face form (a * (u+ - u-)) regrouped per cell, with
//    its conditioning, and no face pass is needed;
//  - expanded (MOL_FLAG_EXPAND_STENCILS): every tap with a variable part, the centre
//    included, is one multiply-add with its per-cell coefficient — the canonical sum, one
//    coefficient per distinct unknown, that ModelingToolkit's compiled f! uses.  Fewer FP64
//    operations; the rounding error relative to the result grows as the sum cancels (like
//    (dx^2 u''/u)^-1 for a diffusion term), so it is a per-plan option.
// Batches (which have no coefficient arrays) take every member's original statements.
struct FoldPart {
    int term;      // member term
    int m;         // interior weight index (MIXED: x * L2 + y; NONLINLAP: outer face 0 or 1)
    double coef;   // the constant, sign included (NONLINLAP: times W and the face's sign)
    int face = -1; // NONLINLAP: the outer face (0: lower, 1: upper) whose a(x) scales coef; -1: constant
};
struct FoldTap {
    int o[3];
    std::vector<FoldPart> parts;
    int arr = -1;        // per-cell coefficient array (index within the group), -1: uniform weight
    bool diff = false;   // difference form: applied to (u[tap] - u[centre])
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
    bool variable = false;                  // has coordinate-dependent (nonlinear-Laplacian) members
    int arr0 = 0;                           // first coefficient array of the group (plan-wide index)
    int narr = 0;                           // coefficient arrays of the group
    // expanded form: an addend quad_sign * k * u^2 of the output (k uniform, u the group's field
    // at the cell) joins the centre tap as (c_0 + quad_sign * k * u) * u; quad_coef is k's pc
    int quad_coef = -1;
    double quad_sign = 0.0;
};
std::vector<FoldGroup> const_linear_groups(const mol_problem_desc* d);
// The fused weights of a group, one per tap: the sum over its constant parts of coefficient *
// weight; in the difference form the centre's entry also holds the differenced taps' constant
// parts.  Taps with a coefficient array hold only their constant parts (k_coef_t adds the rest).
std::vector<double> fold_weights(const mol_problem_desc* d, const FoldGroup& g);
// Coefficient arrays of all groups of a descriptor (the plan allocates [count][ncell]).
int fold_coef_arrays(const std::vector<FoldGroup>& groups);
// True when every nonlinear-Laplacian term of the descriptor is a variable member of some group
// (the face pass then serves only cells off the groups' fast path, which evaluate their faces).
bool nonlinlap_all_in_groups(const mol_problem_desc* d, const std::vector<FoldGroup>& groups);
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
