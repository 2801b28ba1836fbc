// Launcher bodies, instantiated per storage type by step_<type>.cu (the time
// step itself by step_<type>_<parity>.cu).
#pragma once

#include "launch.h"

namespace plbgpu {

// initializeAtEquilibrium (dataInitializerWrapper3D.h:122-130 and
// core/cell.hh iniCellAtEquilibrium): j = u * rho, f-bar_i = the cell's
// computeEquilibrium(i, rho - 1, j, |j|^2); bounce-back and no-dynamics
// cells return 0 (core/dynamics.hh:797-801).
template <typename S, bool ODD>
__global__ void equilibriumKernel(DevLattice L, Box b, const double* rhou, double c0, double c1,
                                  double c2, double c3, double invRho0) {
    using R = typename StoreT<S>::R;
    const int bnz = b.z1 - b.z0 + 1, bny = b.y1 - b.y0 + 1;
    const int dz = blockIdx.x * blockDim.x + threadIdx.x;
    if (dz >= bnz) return;
    const int z = b.z0 + dz, y = b.y0 + blockIdx.y, x = b.x0 + blockIdx.z;
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    const int k = L.flags[idx];
    if (k == K_NONE) return;
    double rho = c0, ux = c1, uy = c2, uz = c3;
    if (rhou) {
        const long long o = (((long long)blockIdx.z * bny + blockIdx.y) * bnz + dz) * 4;
        rho = rhou[o]; ux = rhou[o + 1]; uy = rhou[o + 2]; uz = rhou[o + 3];
    }
    R j[3] = {(R)ux * (R)rho, (R)uy * (R)rho, (R)uz * (R)rho};
    R jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    R rhoBar = (R)rho - (R)1;
    R invRho = (k == K_INCBGK) ? (R)invRho0 : invRhoOf(rhoBar);
    Neighbourhood nb = neighbourhood(L, x, y, z);
    S* Pp = static_cast<S*>(L.pop);
    const bool zero = (k == K_BB || k == K_MEBB || k == K_NODYN);
#pragma unroll
    for (int i = 0; i < 19; ++i) {
        R v = zero ? R(0) : bgkEq<R>(i, rhoBar, invRho, j, jSqr);
        StoreT<S>::st(Pp + slotOf<ODD>(L, nb, idx, i), v);
    }
}

// One time step of the given AA parity.  Each (storage type, parity) pair is
// instantiated in its own translation unit (step_<type>_even.cu /
// step_<type>_odd.cu, from step_parity.cuh) so that the row kernels, the
// costliest code to compile, build in parallel.
template <typename S, bool ODD>
int stepParity(const DevLattice& L, bool stats, const StepParams<typename StoreT<S>::R>& p, StatsAcc* acc,
               cudaStream_t s, const SideStream* side);
// One step of the slab x0 <= x <= x1: its interior rows with the interior-row
// kernels on s, its border rows beside them on the side stream.
template <typename S, bool ODD>
int slabParity(const DevLattice& L, bool stats, const StepParams<typename StoreT<S>::R>& p, StatsAcc* acc, int x0,
               int x1, cudaStream_t s, const SideStream* side);

template <typename S>
struct LaunchImpl {
    using R = typename StoreT<S>::R;
    static constexpr int kBlock = 128;

    static int slabStep(const DevLattice& L, bool odd, bool stats, const StepConsts& c, StatsAcc* acc, int x0, int x1,
                        cudaStream_t s, const SideStream* side) {
        const StepParams<R> p = params(c);
        return odd ? slabParity<S, true>(L, stats, p, acc, x0, x1, s, side)
                   : slabParity<S, false>(L, stats, p, acc, x0, x1, s, side);
    }
    static StepParams<R> params(const StepConsts& c) {
        StepParams<R> p;
        p.bgk.omega = (R)c.omega;
        p.bgk.one_m_omega = (R)c.one_m_omega;
        p.bgk.t0_omega = (R)c.t0_omega;
        p.bgk.t1_omega = (R)c.t1_omega;
        p.bgk.t4_omega = (R)c.t4_omega;
        p.invRho0 = (R)c.invRho0;
        p.pending = c.pending;
        p.seed = c.seed;
        p.external = c.external;
        return p;
    }
    static int step(const DevLattice& L, bool odd, bool stats, const StepConsts& c, StatsAcc* acc,
                    cudaStream_t s, const SideStream* side) {
        const StepParams<R> p = params(c);
        return odd ? stepParity<S, true>(L, stats, p, acc, s, side) : stepParity<S, false>(L, stats, p, acc, s, side);
    }
    static int completeFaces(const DevLattice& L, bool odd, cudaStream_t s) {
        dim3 g = rowGrid(L.nz, L.ny, L.nx, kBlock);
        if (odd) completeFacesKernel<S, true><<<g, kBlock, 0, s>>>(L);
        else completeFacesKernel<S, false><<<g, kBlock, 0, s>>>(L);
        return 1;
    }
    template <typename B>
    static int extractT(const DevLattice& L, bool odd, Box b, int pending, B* out, cudaStream_t s) {
        dim3 g = rowGrid(b.z1 - b.z0 + 1, b.y1 - b.y0 + 1, b.x1 - b.x0 + 1, kXferCells);
        if (odd) extractKernel<S, true, B><<<g, kXferCells, 0, s>>>(L, b, pending, out);
        else extractKernel<S, false, B><<<g, kXferCells, 0, s>>>(L, b, pending, out);
        return 1;
    }
    template <typename B>
    static int insertT(const DevLattice& L, bool odd, Box b, const B* in, cudaStream_t s) {
        dim3 g = rowGrid(b.z1 - b.z0 + 1, b.y1 - b.y0 + 1, b.x1 - b.x0 + 1, kXferCells);
        if (odd) insertKernel<S, true, B><<<g, kXferCells, 0, s>>>(L, b, in);
        else insertKernel<S, false, B><<<g, kXferCells, 0, s>>>(L, b, in);
        return 1;
    }
    static int extract(const DevLattice& L, bool odd, Box b, int pending, double* out, cudaStream_t s) {
        return extractT<double>(L, odd, b, pending, out, s);
    }
    static int insert(const DevLattice& L, bool odd, Box b, const double* in, cudaStream_t s) {
        return insertT<double>(L, odd, b, in, s);
    }
    static int extractF32(const DevLattice& L, bool odd, Box b, int pending, float* out, cudaStream_t s) {
        return extractT<float>(L, odd, b, pending, out, s);
    }
    static int insertF32(const DevLattice& L, bool odd, Box b, const float* in, cudaStream_t s) {
        return insertT<float>(L, odd, b, in, s);
    }
    static int reduce(const DevLattice& L, bool odd, Box b, int pending, double invRho0, double bbRho,
                      ReduceAcc* acc, cudaStream_t s) {
        dim3 g = rowGrid(b.z1 - b.z0 + 1, b.y1 - b.y0 + 1, b.x1 - b.x0 + 1, kBlock);
        if (odd) reduceKernel<S, true><<<g, kBlock, 0, s>>>(L, b, pending, (R)invRho0, bbRho, acc);
        else reduceKernel<S, false><<<g, kBlock, 0, s>>>(L, b, pending, (R)invRho0, bbRho, acc);
        return 1;
    }
    static int field(const DevLattice& L, bool odd, Box b, int pending, double invRho0, double bbRho, int what,
                     double* out, cudaStream_t s) {
        dim3 g = rowGrid(b.z1 - b.z0 + 1, b.y1 - b.y0 + 1, b.x1 - b.x0 + 1, kBlock);
        if (odd) fieldKernel<S, true><<<g, kBlock, 0, s>>>(L, b, pending, (R)invRho0, bbRho, what, out);
        else fieldKernel<S, false><<<g, kBlock, 0, s>>>(L, b, pending, (R)invRho0, bbRho, what, out);
        return 1;
    }
    static int equilibrium(const DevLattice& L, bool odd, Box b, const double* rhou, const double* cst,
                           double invRho0, cudaStream_t s) {
        dim3 g = rowGrid(b.z1 - b.z0 + 1, b.y1 - b.y0 + 1, b.x1 - b.x0 + 1, kBlock);
        if (odd)
            equilibriumKernel<S, true><<<g, kBlock, 0, s>>>(L, b, rhou, cst[0], cst[1], cst[2], cst[3], invRho0);
        else
            equilibriumKernel<S, false><<<g, kBlock, 0, s>>>(L, b, rhou, cst[0], cst[1], cst[2], cst[3], invRho0);
        return 1;
    }
    static int rhoBarJ(const DevLattice& L, bool odd, int pending, double bbRho, cudaStream_t s) {
        using F = typename StoreT<S>::F;
        F* out = static_cast<F*>(const_cast<void*>(L.ext));
        dim3 g = rowGrid(L.nz, L.ny, L.nx, kBlock);
        if (odd) rhoBarJKernel<S, true><<<g, kBlock, 0, s>>>(L, pending, bbRho, out);
        else rhoBarJKernel<S, false><<<g, kBlock, 0, s>>>(L, pending, bbRho, out);
        return 1;
    }
    static int surface(const DevLattice& L, bool odd, const int4* cells, int count, int pending, double invRho0,
                       double bbRho, double omega, cudaStream_t s) {
        if (count <= 0) return 0;
        const int tpb = 64, blocks = (count + tpb - 1) / tpb;
        if (odd)
            surfaceKernel<S, true><<<blocks, tpb, 0, s>>>(L, cells, count, pending, (R)invRho0, bbRho, (R)omega);
        else
            surfaceKernel<S, false><<<blocks, tpb, 0, s>>>(L, cells, count, pending, (R)invRho0, bbRho, (R)omega);
        return 1;
    }
    static int completeFaceList(const DevLattice& L, bool odd, const int4* cells, int count, cudaStream_t s) {
        if (count <= 0) return 0;
        const unsigned blocks = (unsigned)((count + kBlock - 1) / kBlock);
        if (odd) completeFaceListKernel<S, true><<<blocks, kBlock, 0, s>>>(L, cells, count);
        else completeFaceListKernel<S, false><<<blocks, kBlock, 0, s>>>(L, cells, count);
        return 1;
    }
    static const Launchers& table() {
        static const Launchers t = {step,  completeFaces, extract, insert, reduce,
                                    equilibrium, field, rhoBarJ, surface, extractF32, insertF32,
                                    completeFaceList, slabStep};
        return t;
    }
};

}  // namespace plbgpu
