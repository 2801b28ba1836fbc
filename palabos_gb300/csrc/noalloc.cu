// Allocation-free variant of the average energy / density reduction.
//
// Who needs it: callers that own all device memory themselves and may not
// call cudaMalloc -- applications with their own pooled allocator or a fixed
// device-memory budget, and hosts that drive the GPU from a context where
// the runtime allocator is off limits.  They pass the lattice (FP64 f-bar
// planes and cell kinds) and the result buffer; this entry point adds
// nothing to the device heap.
//
// Scratch: one row-sum pair per (x, y) row lives in a file-scope device array
// of NOALLOC_MAX_ROWS entries (4 MiB).  Every GPU that loads this library
// keeps that array until the process exits.  All calls share it: each call
// overwrites the rows it uses before reading them, so nothing carries over,
// but two calls whose kernels overlap on the GPU (different streams, no
// ordering between them) race on the array and may return wrong sums.
//
// Set-up: the device address of the array is looked up once per device, on
// the first call made with that device current (cudaGetSymbolAddress, which
// may also load the module).  Make that first call before any stream capture
// begins.  The address is kept for the life of the process: after a
// cudaDeviceReset of that device the entry point must not be called again.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/plbgpu.h"
#include "d3q19.cuh"

namespace {

constexpr int kMaxRows = PLBGPU_NOALLOC_MAX_ROWS;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_rowSums[2 * kMaxRows];

double* g_rowSumsAddr[kMaxDevices];
bool g_rowSumsReady[kMaxDevices];
std::mutex g_setupMutex;

// First pass: one block per (x, y) row writes that row's sum of |u|^2 and of
// rho-bar.  The per-cell quantities follow computeVelocity / computeRhoBar of
// each dynamics (dataAnalysisFunctional3D.hh:57-123), as in the allocating
// reduction of kernels.cuh.
__global__ void rowSumsKernel(const double* __restrict__ pop, long long stride, const uint8_t* __restrict__ kinds,
                              int nx, int ny, int nz, double bbRhoBar, double invRho0, double* rows) {
    using namespace plbgpu;
    const int row = blockIdx.x;
    const long long base = (long long)row * nz;
    double e = 0., r = 0.;
    bool bad = false;
    for (int z = threadIdx.x; z < nz; z += blockDim.x) {
        const long long idx = base + z;
        const int k = kinds[idx];
        double f[19];
#pragma unroll
        for (int i = 0; i < 19; ++i) f[i] = pop[i * stride + idx];
        double u[3] = {0., 0., 0.}, rb = 0.;
        if (k == K_BGK) {
            double jj[3], rr;
            rhoBarJ<double>(f, rr, jj);
            rb = rhoBarSeq<double>(f);
            double invRho = invRhoOf(rb);
            for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho;
        } else if (k == K_INCBGK) {
            double jj[3], rr;
            rhoBarJ<double>(f, rr, jj);
            for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho0;
            rb = rhoBarSeq<double>(f);
        } else if (k == K_BB || k == K_MEBB) {
            rb = bbRhoBar;
        } else if (k == K_NODYN) {
            rb = 0.;
        } else {
            bad = true;   // kinds that need face values or a force field
        }
        e += u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        r += rb;
    }
    __shared__ double se[32], sr[32];
    __shared__ int sbad;
    if (threadIdx.x == 0) sbad = 0;
    __syncthreads();
    if (bad) atomicOr(&sbad, 1);
    for (int o = 16; o > 0; o >>= 1) {
        e += __shfl_down_sync(0xffffffffu, e, o);
        r += __shfl_down_sync(0xffffffffu, r, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { se[w] = e; sr[w] = r; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double te = 0., tr = 0.;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { te += se[i]; tr += sr[i]; }
        if (sbad) te = tr = __longlong_as_double(0x7ff8000000000000ll);   // NaN: unsupported kind
        rows[2 * row] = te;
        rows[2 * row + 1] = tr;
    }
}

// Second pass: one block sums the row pairs in a fixed order and writes the
// two averages.
__global__ void finishKernel(const double* rows, int nrows, double cells, double* result) {
    __shared__ double se[1024], sr[1024];
    double e = 0., r = 0.;
    for (int i = threadIdx.x; i < nrows; i += blockDim.x) {
        e += rows[2 * i];
        r += rows[2 * i + 1];
    }
    se[threadIdx.x] = e;
    sr[threadIdx.x] = r;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            se[threadIdx.x] += se[threadIdx.x + s];
            sr[threadIdx.x] += sr[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        result[0] = se[0] / 2.0 / cells;     // getSumEnergy() / nCells
        result[1] = sr[0] / cells + 1.0;     // fullRho(sumRhoBar / nCells)
    }
}

// Device address of the scratch array for the current device.
int scratchForCurrentDevice(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PLBGPU_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return PLBGPU_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_setupMutex);
    if (!g_rowSumsReady[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_rowSums) != cudaSuccess || !p) return PLBGPU_ERR_CUDA;
        g_rowSumsAddr[dev] = static_cast<double*>(p);
        g_rowSumsReady[dev] = true;
    }
    *out = g_rowSumsAddr[dev];
    return PLBGPU_OK;
}

}  // namespace

extern "C" int plbgpu_reduce_noalloc(const double* populations, long long stride, const uint8_t* kinds, int nx,
                                     int ny, int nz, double bb_rho, double rho0, double* result, void* stream) {
    if (!populations || !kinds || !result || nx < 1 || ny < 1 || nz < 1) return PLBGPU_ERR_ARG;
    if ((long long)nx * ny > kMaxRows) return PLBGPU_ERR_ARG;         // more rows than the scratch holds
    if (stride < (long long)nx * ny * nz || !(rho0 != 0.0)) return PLBGPU_ERR_ARG;
    double* rows = nullptr;
    int rc = scratchForCurrentDevice(&rows);
    if (rc != PLBGPU_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int nrows = nx * ny;
    rowSumsKernel<<<nrows, 128, 0, s>>>(populations, stride, kinds, nx, ny, nz, bb_rho - 1.0, 1.0 / rho0, rows);
    if (cudaGetLastError() != cudaSuccess) return PLBGPU_ERR_CUDA;
    finishKernel<<<1, 1024, 0, s>>>(rows, nrows, (double)nx * ny * nz, result);
    if (cudaGetLastError() != cudaSuccess) return PLBGPU_ERR_CUDA;
    return PLBGPU_OK;
}
