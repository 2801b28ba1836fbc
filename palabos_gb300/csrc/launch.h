// Host-side launchers of the lattice kernels, one set per storage precision.
// The FP64 set lives in a translation unit compiled without FMA contraction
// (bit-exact with the reference); the FP32 / BF16 / FP16 sets in one compiled
// with contraction.
#pragma once

#include <cuda_runtime.h>

#include "kernels.cuh"

namespace plbgpu {

struct StepConsts {
    double omega, one_m_omega, t0_omega, t1_omega, t4_omega;
    double invRho0;
    int pending;
    unsigned seed;
    int external;   // collide with the external rho-bar / j planes (DevLattice::ext)
};

// A second stream for the border rows of a step: they touch no population
// slot of the interior rows in the same step, so the two kernels run
// concurrently (fork and join through the two events).
struct SideStream {
    cudaStream_t stream;
    cudaEvent_t fork, join;
};

// Each launcher returns the number of kernels it launched.
struct Launchers {
    int (*step)(const DevLattice&, bool odd, bool stats, const StepConsts&, StatsAcc*, cudaStream_t,
                const SideStream*);
    int (*completeFaces)(const DevLattice&, bool odd, cudaStream_t);
    int (*extract)(const DevLattice&, bool odd, Box, int pending, double* out, cudaStream_t);
    int (*insert)(const DevLattice&, bool odd, Box, const double* in, cudaStream_t);
    int (*reduce)(const DevLattice&, bool odd, Box, int pending, double invRho0, double bbRho,
                  ReduceAcc*, cudaStream_t);
    int (*equilibrium)(const DevLattice&, bool odd, Box, const double* rhou, const double* cst,
                       double invRho0, cudaStream_t);
    int (*field)(const DevLattice&, bool odd, Box, int pending, double invRho0, double bbRho, int what,
                 double* out, cudaStream_t);
    // BoxRhoBarJfunctional3D into the external planes (DevLattice::ext).
    int (*rhoBarJ)(const DevLattice&, bool odd, int pending, double bbRho, cudaStream_t);
    // Edge or corner cells (x, y, z, kind) finished after a step.
    int (*surface)(const DevLattice&, bool odd, const int4* cells, int count, int pending, double invRho0,
                   double bbRho, double omega, cudaStream_t);
    // The transfer layout with FP32 records (the single-precision co-processor form).
    int (*extractF32)(const DevLattice&, bool odd, Box, int pending, float* out, cudaStream_t);
    int (*insertF32)(const DevLattice&, bool odd, Box, const float* in, cudaStream_t);
    // Face cells (x, y, z, kind) of interior rows completed in place before a step.
    int (*completeFaceList)(const DevLattice&, bool odd, const int4* cells, int count, cudaStream_t);
    // One step of the slab x0 <= x <= x1 only, for steps pipelined with transfers (border rows on the
    // side stream when one is given).
    int (*slabStep)(const DevLattice&, bool odd, bool stats, const StepConsts&, StatsAcc*, int x0, int x1,
                    cudaStream_t, const SideStream*);
};

const Launchers& launchersFp64();
const Launchers& launchersFp32();
const Launchers& launchersBf16();
const Launchers& launchersFp16();
const Launchers& launchersBf16Sr();

}  // namespace plbgpu

struct plbgpu_ctx;

namespace plbgpu {

// A domain as the adjoint module sees it (implemented in api.cu).
struct DomainAccess {
    DevLattice L;
    int precision;
    bool odd, pending;
    double omega, rho0, bbRho;
    cudaStream_t stream;
    void** adjointSlot;            // per-domain storage owned by the adjoint module
    void (**adjointFree)(void*);   // its release function, called when the domain goes away
    unsigned long long* launches;  // the context's kernel-launch counter
};
int domainAccess(plbgpu_ctx* c, int handle, DomainAccess* out);
int domainFail(plbgpu_ctx* c, int code, const char* msg);
// The context's stream (kernels that belong to no domain, e.g. the voxelizer).
cudaStream_t contextStream(plbgpu_ctx* c);
// Add n kernel launches to the context's counter.
void countLaunches(plbgpu_ctx* c, int n);
// After the adjoint module rewrote the populations in natural order.
void domainSetState(plbgpu_ctx* c, int handle, bool odd, bool pending);
// The domain's checked list of external velocity edge cells, then corner
// cells (x, y, z, kind), rebuilt first when the kinds changed.
int domainSurface(plbgpu_ctx* c, int handle, const int4** cells, int* nEdges, int* nCorners);

// Binary-block checkpoints (checkpoint.cu): base64 of the byte stream
// head[0..headLen) ++ body[0..bodyLen) as `quads` output quads (the last one
// padded when the stream ends inside it), the inverse, and a column copy
// between packed per-cell records.
void launchBase64Encode(const uint8_t* head, int headLen, const uint8_t* body, size_t bodyLen, size_t quads,
                        char* out, cudaStream_t s);
void launchBase64Decode(const char* in, size_t quads, size_t bytes, uint8_t* out, unsigned* bad, cudaStream_t s);
void launchColumns(const double* in, int inStride, int inOff, int m, double* out, int outStride, int outOff,
                   long long cells, cudaStream_t s);

inline dim3 rowGrid(int nz, int ny, int nx, int block) {
    return dim3((unsigned)((nz + block - 1) / block), (unsigned)ny, (unsigned)nx);
}

}  // namespace plbgpu
