// FP64 pipe rate of the GPU, measured by the library itself: the FP64 form of
// the step is bound by the FP64 pipe (every add and multiply of the
// reference's collision rounded separately, no FMA contraction), so its
// roofline is this rate, not HBM bandwidth.
//
// Each thread runs kChains independent dependency chains of one DMUL and one
// DADD per iteration (the translation unit is compiled with --fmad=false, so
// the pair is not contracted into a DFMA), enough independent work per SM to
// keep the pipe busy.  Ops counted = adds + multiplies.
#include <cuda_runtime.h>

#include "../../include/plbgpu.h"
#include "launch.h"

namespace {

constexpr int kChains = 16;
constexpr int kIters = 1024;
constexpr int kThreads = 256;
constexpr int kBlocksPerSm = 8;

__global__ void __launch_bounds__(kThreads) fp64ChainKernel(double* out, double m, double c) {
    double a[kChains];
#pragma unroll
    for (int k = 0; k < kChains; ++k) a[k] = 1.0 + 1e-3 * (double)(threadIdx.x + k);
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int k = 0; k < kChains; ++k) {
            a[k] = a[k] * m;
            a[k] = a[k] + c;
        }
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < kChains; ++k) s += a[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;   // keeps the chains live
}

}  // namespace

extern "C" int plbgpu_measure_fp64_rate(plbgpu_ctx* c, double* ops_per_second) {
    if (!c || !ops_per_second) return PLBGPU_ERR_ARG;
    cudaStream_t s = plbgpu::contextStream(c);
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return plbgpu::domainFail(c, PLBGPU_ERR_CUDA, "fp64 rate: device query failed");
    const int grid = sms * kBlocksPerSm;
    double* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaMalloc(&out, sizeof(double) * (size_t)grid * kThreads) != cudaSuccess)
        return plbgpu::domainFail(c, PLBGPU_ERR_NOMEM, "fp64 rate: device allocation failed");
    int rc = PLBGPU_OK;
    float best = 0.f;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        rc = plbgpu::domainFail(c, PLBGPU_ERR_CUDA, "fp64 rate: event creation failed");
    } else {
        // one untimed launch, then the fastest of three
        for (int r = 0; r < 4 && rc == PLBGPU_OK; ++r) {
            cudaEventRecord(e0, s);
            fp64ChainKernel<<<grid, kThreads, 0, s>>>(out, 0.999999, 1e-7);
            plbgpu::countLaunches(c, 1);
            cudaEventRecord(e1, s);
            if (cudaGetLastError() != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
                rc = plbgpu::domainFail(c, PLBGPU_ERR_CUDA, "fp64 rate: kernel failed");
                break;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (r > 0 && (best == 0.f || ms < best)) best = ms;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    if (rc) return rc;
    const double ops = (double)grid * kThreads * kIters * kChains * 2.0;
    *ops_per_second = ops / ((double)best * 1e-3);
    return PLBGPU_OK;
}
