// Device diagnostics behind the design of the kernels (not on the solve path).
//
// mol_diag_fp64_rate measures the FP64 pipe on the current device: every warp of a grid of
// (SMs x 4) CTAs x 256 threads runs eight independent FMA chains on `active` of its 32 lanes.
// On GB300 the time does not depend on `active`: an FP64 warp instruction costs the same
// however few lanes are active, which is why the generated kernels keep warps converged
// around FP64 arithmetic instead of splitting lanes between paths.
#include <cuda_runtime.h>

#include "mol_plan.h"

namespace {

__global__ void k_fp64_chains(double* out, int iters, int active) {
    const int lane = threadIdx.x & 31;
    double a0 = threadIdx.x * 1e-9, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3;
    double a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6, a7 = a0 + 7;
    const double m = 0.999999, c = 1e-7;
    if (lane < active) {
        for (int i = 0; i < iters; ++i) {
            a0 = fma(a0, m, c);
            a1 = fma(a1, m, c);
            a2 = fma(a2, m, c);
            a3 = fma(a3, m, c);
            a4 = fma(a4, m, c);
            a5 = fma(a5, m, c);
            a6 = fma(a6, m, c);
            a7 = fma(a7, m, c);
        }
    }
    out[blockIdx.x * (long long)blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

}  // namespace

extern "C" {

int mol_diag_fp64_rate(int32_t active_lanes, double* warp_fma_per_s, double* lane_tflops) {
    if (active_lanes < 1 || active_lanes > 32 || !warp_fma_per_s) return MOL_ERR_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                   cudaSuccess) {
        cudaGetLastError();
        return MOL_ERR_CUDA;
    }
    const int blocks = sms * 4, threads = 256, iters = 4096;
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double) * (size_t)blocks * threads) != cudaSuccess) {
        cudaGetLastError();
        return MOL_ERR_OOM;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fp64_chains<<<blocks, threads>>>(out, iters, active_lanes);  // warm-up
    cudaEventRecord(e0);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) k_fp64_chains<<<blocks, threads>>>(out, iters, active_lanes);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return MOL_ERR_CUDA;
    const double sec = ms * 1e-3 / reps;
    const double warp_fma = (double)blocks * threads / 32 * iters * 8;
    *warp_fma_per_s = warp_fma / sec;
    if (lane_tflops) *lane_tflops = 2.0 * warp_fma * active_lanes / sec / 1e12;
    return MOL_OK;
}

}  // extern "C"
