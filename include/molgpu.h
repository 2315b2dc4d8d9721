/*
 * molgpu — GB300 (sm_103a) method-of-lines hot path behind a C ABI.
 *
 * This library replaces the runtime hot path that MethodOfLines.jl hands to
 * ModelingToolkit and OrdinaryDiffEq: the generated semi-discrete right-hand
 * side f!(du, u, p, t) and the explicit time steppers that call it.  The
 * symbolic front end (PDEBase/MethodOfLines rule generation) stays on the host
 * and lowers a PDE system into the plain-data `mol_problem_desc` below; the
 * library owns all device memory of a plan and every kernel.
 *
 * Conventions
 *  - The unknown vector has the layout of the reference's `unknowns(simpsys)`:
 *    fields in declaration order, each field's interior box flattened with the
 *    first spatial dimension fastest (docs/src/generated/bruss_code.md).
 *  - Grid indices in the descriptor are 1-based like Julia's; npts[d] counts
 *    every grid point of dimension d, boundary points included.
 *  - Pointers passed to the solver entry points may be host or device memory;
 *    the library detects which (cudaPointerGetAttributes) and copies host
 *    buffers in and out around the call.
 *  - Every entry point returns a mol_status (0 = success).  No exception, abort
 *    or device trap crosses the ABI; mol_last_error() describes the failure.
 *  - A plan is bound to the device that was current at creation and to one
 *    CUDA stream (its own unless mol_plan_set_stream is called).  A plan is not
 *    thread-safe; distinct plans are independent.
 */
#ifndef MOLGPU_H
#define MOLGPU_H

#ifndef __CUDACC_RTC__
#include <stdint.h>
#else
/* runtime compilation (NVRTC) of the generated right-hand side sees this header too */
typedef signed char int8_t;
typedef short int16_t;
typedef int int32_t;
typedef long long int64_t;
typedef unsigned short uint16_t;
typedef unsigned int uint32_t;
typedef unsigned long long uint64_t;
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define MOL_ABI_VERSION 2
#define MOL_MAX_DIMS 3
#define MOL_MAX_FIELDS 8
#define MOL_MAX_REGS 64

typedef enum mol_status {
    MOL_OK = 0,
    MOL_ERR_INVALID = -1,       /* malformed descriptor or argument            */
    MOL_ERR_OOM = -2,           /* device allocation failed                     */
    MOL_ERR_NONFINITE = -3,     /* NaN/Inf in the state or the step size        */
    MOL_ERR_TIMEOUT = -4,       /* a bounded device wait ran out                */
    MOL_ERR_CUDA = -5,          /* CUDA runtime error (text in mol_last_error)  */
    MOL_ERR_UNSUPPORTED = -6,   /* term/boundary combination not implemented    */
    MOL_ERR_MAXITERS = -7,      /* adaptive solver hit its iteration limit      */
    MOL_ERR_DTMIN = -8          /* adaptive step size underflowed               */
} mol_status;

/* ------------------------------------------------------------------------ */
/* Problem descriptor                                                       */
/* ------------------------------------------------------------------------ */

/* One 1-D derivative operator: the reference's DerivativeOperator
 * (src/discretization/derivative_operator.jl:1-15) with its tap-selection rule
 * (centered_difference.jl:5-30, upwind_difference.jl:1-28,
 * half_offset_centred_difference.jl:9-37).  For a point i along a dimension of
 * `len` points:
 *   i <= nlo (non-periodic)        -> low table i-1, taps 1 .. bLlo
 *   i >  len - nhi (non-periodic)  -> high table (len - i - hi_base), taps len-bLhi+1 .. len
 *   otherwise                      -> interior weights, taps i+omin .. i+omin+L-1 (wrapped if periodic)
 * Weights are offsets into mol_problem_desc.weights.  nrows = 0: one interior row shared by
 * every interior point.  nrows > 0 (a nonuniform grid, centered_diff_weights.jl:77-153 and
 * the DX <: AbstractVector method of centered_difference.jl:32-56): one row of L weights per
 * interior point, row (i - nlo - 1) at w_int + (i - nlo - 1) * L; then every interior
 * position that reads an interior row needs one (nrows >= min(len - upper, len - nhi) - nlo),
 * the dimension must not be periodic, and only LINEAR terms may use the operator
 * (MOL_ERR_UNSUPPORTED otherwise).  The reference's nonuniform upwind operators
 * (upwind_diff_weights.jl:93-171 with the selection of upwind_difference.jl:131-162) are
 * expressed this way too. */
typedef struct mol_op1d {
    int32_t L, omin, nlo, bLlo, nhi, bLhi, hi_base, nrows;
    int64_t w_int, w_lo, w_hi;
} mol_op1d;

typedef enum mol_term_kind {
    MOL_TERM_LINEAR = 1,    /* sum_k w_k u[tap_k] along `dim` (centered or upwind)      */
    MOL_TERM_MIXED = 2,     /* sum_ab wa wb u[tap_a, tap_b] (2nd_order_mixed_deriv.jl)  */
    MOL_TERM_WENO = 3,      /* Jiang-Shu WENO5 node derivative (WENO.jl:6-57)           */
    MOL_TERM_NONLINLAP = 4  /* Dx(a(x,u) Dx u) (nonlinear_laplacian.jl:28-103)          */
} mol_term_kind;

typedef struct mol_term {
    int32_t kind;
    int32_t field;      /* differentiated field                                        */
    int32_t dim, dim2;  /* dimension(s), 0-based                                        */
    int32_t op, op2, op3; /* LINEAR: op. MIXED: op (dim), op2 (dim2).
                           NONLINLAP: op = outer half-offset d1, op2 = inner half-offset d1,
                           op3 = half-offset interpolation (order 0).
                           WENO with variant 1: op holds the per-point geometry rows      */
    int32_t prog;       /* NONLINLAP: face program (outputs a at the half point)        */
    int32_t aux0;       /* NONLINLAP: first face-aux array used by the face program      */
    int32_t reserved0;  /* filled by the library                                         */
    int32_t variant;    /* WENO: 0 uniform Jiang-Shu (WENO.jl:6-57); 1 node-centred Lagrange
                           WENO-5 on a nonuniform dimension (nonuniform_weno.jl:1-212): op's
                           row i-1 (nrows = npts, L = 56) holds point i's geometry: dx/6, dx,
                           dx^3, per substencil the first-derivative weights at the target,
                           the Simpson cell's ends and middle and the second-derivative
                           weights at the middle, then dp_k/sigma_p, dm_k/sigma_m, sigma_p,
                           sigma_m; taps 1..5 (points 1, 2), n-4..n (points n-1, n) or
                           i-2..i+2                                                       */
    int32_t reserved2;
    double eps;         /* WENO epsilon                                                  */
    double dx;          /* WENO grid spacing                                             */
} mol_term;

typedef enum mol_bc_kind {
    MOL_BC_NONE = 0,      /* no boundary row on this face (interior extends to the end)     */
    MOL_BC_PERIODIC = 1,  /* u[1] ~ u[l] (generate_bc_eqs.jl:35-58, interface_boundary.jl:33-42) */
    MOL_BC_ROBIN = 2,     /* a*u + b*Dx(u) = g at the face, solved for the boundary value     */
    MOL_BC_EDGE = 3       /* edge-aligned grid: a*I(u) + b*H(u) = g at the face half-way between
                             the ghost point and the first (last) unknown, I the interpolation
                             table `iop` and H the half-offset first-derivative table `op` at
                             position 1 (n-1), solved for the ghost point (boundary_value_maps for
                             EdgeAlignedGrid, generate_bc_eqs.jl:80-160)                       */
} mol_bc_kind;

typedef struct mol_bc {
    int32_t kind;
    int32_t prog;       /* -1: a,b,g below are constants; else program with outputs 0:a 1:b 2:g */
    int32_t op;         /* centered first-derivative operator whose boundary table the row uses */
    int32_t extrap;     /* 0, or 1 + the operator holding the extrapolation table of the point
                           next to this boundary point (generate_extrap_eqs!, generate_bc_eqs.jl:
                           336-392): when the interior stops two points from the end (WENO on a
                           bounded uniform dimension, WENO.jl:94), point 2 (or n-1) is observed as
                           sum_k w_k u[k] over the first (last) bL points with the second low (high)
                           row of that operator, the boundary point through this row, which must
                           then be a Dirichlet row (b == 0)                                     */
    double a, b, g;
    int32_t iop;        /* MOL_BC_EDGE: the half-offset interpolation operator              */
    int32_t pad;
} mol_bc;

/* Register-machine instruction of the pointwise programs. */
typedef struct mol_instr {
    uint16_t op, dst, a, b, c, reserved;
    int32_t imm;
} mol_instr;

typedef enum mol_opcode {
    MOL_OP_CONST = 1,   /* r[dst] = consts[imm]                                  */
    MOL_OP_PARAM,       /* r[dst] = p[imm]                                       */
    MOL_OP_FIELD,       /* r[dst] = field imm at the cell (face: interpolated)    */
    MOL_OP_AUX,         /* r[dst] = aux array imm at the cell (face: at the face) */
    MOL_OP_COORD,       /* r[dst] = grid coordinate of dimension imm             */
    MOL_OP_TIME,        /* r[dst] = t                                            */
    MOL_OP_TERM,        /* r[dst] = derivative term imm at the cell               */
    MOL_OP_UPWIND,      /* r[dst] = r[a] < 0 ? r[a]*T[b] : r[a]*T[c]  (rhs form) */
    MOL_OP_ADD, MOL_OP_SUB, MOL_OP_MUL, MOL_OP_DIV,
    MOL_OP_NEG,         /* r[dst] = -r[a]                                        */
    MOL_OP_POWI,        /* r[dst] = r[a]^imm (x*x, x*x*x, else pow)              */
    MOL_OP_POW,         /* r[dst] = pow(r[a], r[b])                              */
    MOL_OP_FN,          /* r[dst] = fn_imm(r[a])                                  */
    MOL_OP_CMP,         /* r[dst] = (r[a] cmp_imm r[b]) ? 1 : 0                   */
    MOL_OP_IFELSE,      /* r[dst] = r[a] != 0 ? r[b] : r[c]                       */
    MOL_OP_OUT          /* output imm = r[a]                                      */
} mol_opcode;

typedef enum mol_fn { MOL_FN_SIN = 0, MOL_FN_COS, MOL_FN_TAN, MOL_FN_EXP, MOL_FN_LOG,
                      MOL_FN_SQRT, MOL_FN_ABS, MOL_FN_TANH, MOL_FN_SINH, MOL_FN_COSH,
                      MOL_FN_ATAN } mol_fn;
typedef enum mol_cmp { MOL_CMP_LE = 0, MOL_CMP_LT, MOL_CMP_GE, MOL_CMP_GT, MOL_CMP_EQ } mol_cmp;

#define MOL_FLAG_NONE 0
/* Coordinate-dependent linear stencils (a nonlinear Laplacian Dj(K(x) Dj u) whose face
 * coefficient reads only aux arrays and constants, with the first-derivative stencils of
 * constant coefficient beside it in the same output) are evaluated from per-cell coefficient
 * arrays filled once at plan creation.  By default the taps are applied to differences
 * u[tap] - u[cell] (the face form's conditioning); with this flag as one expanded sum
 * sum_k c_k[cell] u[tap_k] (ModelingToolkit's canonical sum: fewer FP64 operations, rounding
 * error that grows with the cancellation of the sum, about (dx^2 u''/u)^-1 for diffusion). */
#define MOL_FLAG_EXPAND_STENCILS 1

typedef struct mol_problem_desc {
    int32_t abi_version;            /* MOL_ABI_VERSION                                   */
    int32_t ndim;                   /* 1..3 spatial dimensions                           */
    int32_t nfields;                /* 1..MOL_MAX_FIELDS dependent variables            */
    int32_t nparams;
    int64_t npts[MOL_MAX_DIMS];     /* grid points per dimension (boundary included)     */
    int32_t lower[MOL_MAX_DIMS];    /* points clipped at the low end (interior_map.jl)   */
    int32_t upper[MOL_MAX_DIMS];    /* points clipped at the high end                    */
    double dx[MOL_MAX_DIMS];
    const double* coords[MOL_MAX_DIMS];   /* npts[d] grid coordinates                   */
    mol_bc bc[MOL_MAX_FIELDS][MOL_MAX_DIMS][2];   /* [field][dim][low=0/high=1]          */
    int32_t nops;      const mol_op1d* ops;
    int64_t nweights;  const double* weights;
    int32_t nterms;    const mol_term* terms;
    int32_t ninstr;    const mol_instr* code;
    int32_t nprogs;    const int32_t* prog_ranges; /* nprogs pairs (start, length)     */
    int32_t cell_prog;                           /* program with one OUT per field     */
    int32_t nconsts;   const double* consts;
    int32_t naux;      const double* const* aux; const int64_t* aux_len;
    const double* params;                        /* default parameter values (nparams) */
    int32_t flags;
    int32_t reserved;
} mol_problem_desc;

typedef struct mol_plan mol_plan;
typedef struct mol_batch mol_batch;

typedef struct mol_stats {
    int64_t naccept, nreject, nf;
    double t, dt;
} mol_stats;

/* ------------------------------------------------------------------------ */
/* Library and plan                                                          */
/* ------------------------------------------------------------------------ */

int mol_version(void);
const char* mol_status_string(int status);

/* Replaces discretize(pdesys, MOLFiniteDifference(...)) -> ODEProblem at the
 * point where ModelingToolkit compiles f! (src/MOL_discretization.jl:171-201).
 * Copies the descriptor and every array it points to. */
int mol_plan_create(const mol_problem_desc* desc, mol_plan** out);
int mol_plan_destroy(mol_plan* plan);
/* generate_code(pdesys, disc) (src/MOL_discretization.jl:208-217): the CUDA source the
 * library generates for this problem structure; needs no device.  `needed` receives
 * the buffer size including the terminating NUL. */
int mol_generate_code(const mol_problem_desc* desc, char* buf, int64_t bufsize, int64_t* needed);
/* Generates and compiles (NVRTC, sm_103a) without loading; needs no device.  `log`
 * receives the compiler log on failure. */
int mol_codegen_compile_check(const mol_problem_desc* desc, char* log, int64_t logsize);
const char* mol_last_error(const mol_plan* plan);
int mol_plan_set_stream(mol_plan* plan, void* cuda_stream);
int64_t mol_plan_n_unknowns(const mol_plan* plan);
/* Kernel launches issued by this process so far (all plans). */
int64_t mol_launch_count(void);
/* 1 when the plan runs the generated (NVRTC-compiled) right-hand side, 0 for the
 * register-machine interpreter; the source text (or the reason it is off). */
int mol_plan_uses_codegen(const mol_plan* plan);
/* Number of per-cell coefficient arrays the plan holds for its coefficient stencils
 * (see MOL_FLAG_EXPAND_STENCILS); 0 when it has none.  Each array holds one value per
 * interior cell and is read once per right-hand-side evaluation.  New entry point: it has no
 * counterpart in the reference, whose compiled f! carries such weights as literals. */
int mol_plan_coef_arrays(const mol_plan* plan);
const char* mol_plan_codegen_source(const mol_plan* plan);
/* Registers per thread of the generated stage kernel (0 for the interpreter), threads per
 * CTA and CTAs of the plan's grid-stride launches. */
int mol_plan_launch_config(const mol_plan* plan, int32_t* regs, int32_t* threads, int32_t* blocks);

/* ------------------------------------------------------------------------ */
/* Hot path                                                                  */
/* ------------------------------------------------------------------------ */

/* f!(du, u, p, t): the generated ODEFunction, called exactly as
 * benchmark/weno/suite.jl:283-289 does.  p may be NULL (descriptor defaults). */
/* Full-grid values of the state u at time t for every field: the unknowns, the observed
 * boundary values (boundary rows, extrapolated points, ghost points of edge-aligned grids), the
 * periodic images (u[1] ~ u[l]) and the corner points (~ 0), field-major with the first
 * dimension fastest, nfields * npts[0] * npts[1] * npts[2] doubles (unused dimensions count 1).
 * Replaces the observed-variable reconstruction behind sol[u(t, x)] of the reference's
 * PDETimeSeriesSolution (src/interface/solution/timedep.jl:19-80).  u, p, full: host or
 * device; a host `full` is written before the call returns. */
int mol_fill_grid(mol_plan* plan, const double* u, const double* p, double t, double* full);

int mol_rhs(mol_plan* plan, double* du, const double* u, const double* p, double t);
int mol_rhs_f32state(mol_plan* plan, float* du, const float* u, const float* p, double t);

/* solve(prob, SSPRK33(); dt, adaptive=false) for nsteps steps from t0, in place on u
 * (OrdinaryDiffEqSSPRK SSPRK33, used at benchmark/weno/suite.jl:291-295).  Every step's
 * result is tested for NaN and Inf on the GPU (OrdinaryDiffEq's default unstable_check,
 * which ends such a solve with ReturnCode.Unstable).  On host state the call waits for the
 * steps and returns MOL_ERR_NONFINITE when one produced such a value; on device state it
 * stays asynchronous and mol_plan_check reports it. */
int mol_step_ssprk33(mol_plan* plan, double* u, const double* p, double t0, double dt, int64_t nsteps);
int mol_step_ssprk33_f32state(mol_plan* plan, float* u, const float* p, double t0, double dt, int64_t nsteps);
/* Waits for the plan's stream and returns MOL_ERR_NONFINITE (then clears the condition) when
 * an SSPRK33 step since the last check, on this plan, produced a NaN or Inf state value. */
int mol_plan_check(mol_plan* plan);
/* Same steps as mol_step_ssprk33, for callers that cannot let the call allocate device
 * memory (a device-memory budget fixed up front, e.g. a pool that must not grow or one
 * GPU divided between several plans at start-up; host callbacks, where CUDA allocation
 * calls are not allowed).  No counterpart in the reference.  The two stage buffers live
 * in one static device array sized for at most 2^20 unknowns (16 MiB, held by every GPU
 * that loads the library until exit); larger plans get MOL_ERR_INVALID, as do host
 * arrays (u and p must be device memory) and non-finite t0 or dt.  The plan's kernels
 * are loaded by mol_plan_create, so the call loads nothing.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) and should come before any
 * stream capture.  All calls share the array: calls that overlap on the GPU race. */
int mol_step_ssprk33_noalloc(mol_plan* plan, double* u, const double* p, double t0, double dt, int64_t nsteps);

/* solve(prob, Tsit5(); abstol, reltol) from t0 to t1, in place on u
 * (test/Burgers/burgers_eq.jl:39).  dt0 <= 0 selects the initial step automatically;
 * maxiters <= 0 allows 10^8 steps.  Non-finite times, tolerances or dt0 give MOL_ERR_INVALID. */
int mol_solve_tsit5(mol_plan* plan, double* u, const double* p, double t0, double t1,
                    double abstol, double reltol, double dt0, int64_t maxiters, mol_stats* stats);

/* Discrete adjoint of nsteps fixed-step SSPRK33 steps.  Loss kinds:
 *   MOL_LOSS_MISFIT:  L = 0.5*||u(T) - target||^2, `target` = target state
 *   MOL_LOSS_LAMBDA:  `target` is dL/du(T) supplied by the caller
 * Outputs (any may be NULL): uT, loss, dL/du0 (n_unknowns), dL/dp (nparams),
 * dL/daux (concatenated aux arrays in descriptor order).  nsnap checkpoints
 * (binomial/revolve schedule) bound the stored states; nsnap <= 0 keeps every state (and both
 * stage values of every step) that fits in three quarters of the free device memory, for the
 * duration of the call.  MOL_ERR_NONFINITE when a forward
 * step produced a NaN or Inf state value (as mol_plan_check) or the loss is not finite. */
#define MOL_LOSS_MISFIT 0
#define MOL_LOSS_LAMBDA 1
int mol_adjoint_ssprk33(mol_plan* plan, const double* u0, const double* p, double t0, double dt,
                        int64_t nsteps, int32_t nsnap, int32_t loss_kind, const double* target,
                        double* uT, double* loss, double* dLdu0, double* dLdp, double* dLdaux,
                        int64_t* nforward_steps);
/* Vector-Jacobian product of the RHS: lam_u = lambda^T df/du, lam_p = lambda^T df/dp,
 * lam_aux = lambda^T df/daux (accumulated into the outputs, which may be NULL). */
int mol_rhs_vjp(mol_plan* plan, const double* lambda, const double* u, const double* p, double t,
                double* lam_u, double* lam_p, double* lam_aux);

/* ------------------------------------------------------------------------ */
/* Batched ensemble: many instances of one PDE structure, uneven grid sizes  */
/* ------------------------------------------------------------------------ */

/* All descriptors must share the term/program structure; grid sizes, spacings,
 * weights, parameters and aux arrays may differ. */
int mol_batch_create(const mol_problem_desc* const* descs, int32_t ninstances, mol_batch** out);
int mol_batch_destroy(mol_batch* batch);
const char* mol_batch_last_error(const mol_batch* batch);
int mol_batch_set_stream(mol_batch* batch, void* cuda_stream);
/* Offsets of each instance in the packed state vector (ninstances + 1 entries). */
int mol_batch_offsets(const mol_batch* batch, int64_t* offsets);
/* One persistent launch advances every instance nsteps SSPRK33 steps with its own dt. */
int mol_batch_step_ssprk33(mol_batch* batch, double* u_packed, const double* dts, double t0, int64_t nsteps);
int mol_batch_step_ssprk33_f32state(mol_batch* batch, float* u_packed, const double* dts, double t0, int64_t nsteps);
/* Tuning: threads per CTA, CTAs per SM and the schedule: tile_cells > 0 splits every
 * stage of every instance into tiles of that many cells (units handed out across the
 * GPU, stages ordered per instance by counters), tile_cells < 0 runs one CTA per
 * instance.  0 leaves a setting as it is; all three 0 autotune again on the next run. */
int mol_batch_tune(mol_batch* batch, int32_t threads, int32_t ctas_per_sm, int64_t tile_cells);
/* Waits for the batch's stream and reports a run that was abandoned because a stage
 * dependency wait ran out of its poll budget (MOL_ERR_CUDA), or a step since the last check
 * that produced a NaN or Inf state value in some instance (MOL_ERR_NONFINITE, OrdinaryDiffEq's
 * unstable_check); the condition is then cleared.  Steps on host arrays call it themselves. */
int mol_batch_check(mol_batch* batch);
/* The schedule in use (after autotuning, once a step has run): threads per CTA, CTAs per SM,
 * tile cells (-1: one CTA per instance). */
int mol_batch_config(const mol_batch* batch, int32_t* threads, int32_t* ctas_per_sm, int64_t* tile_cells);

/* ---- diagnostics (no reference counterpart) ---- */
/* FP64 pipe on the current device: warp-level FMA instructions per second when `active_lanes`
 * (1..32) lanes of every warp run eight independent FMA chains, and the lane-level TFLOP/s
 * (optional).  On GB300 the warp rate does not depend on the number of active lanes. */
int mol_diag_fp64_rate(int32_t active_lanes, double* warp_fma_per_s, double* lane_tflops);

#ifdef __cplusplus
}
#endif
#endif /* MOLGPU_H */
