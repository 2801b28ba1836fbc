// Device kernels of the D3Q19 lattice: fused collide-and-stream in the AA
// pattern, state transfer in the canonical co-processor layout, reductions.
//
// Storage: structure of arrays.  Population i of cell c lives at
// pop[i * stride + c], c = (x * ny + y) * nz + z.  Values are f-bar (f - t_i),
// the reference's own stored representation (roundOffPolicy.h:40-89), in the
// storage type S (double, float, bfloat16 or half).
//
// AA pattern (in place, one array):
//   even step  read slot i of cell x, collide, write f*_i to slot opp(i) of x;
//   odd step   read slot opp(i) of x - c_i, collide, write f*_i to slot i of
//              x + c_i.
// After an odd step the array is in natural order again.  A population whose
// source or destination lies outside a non-periodic domain stays in its own
// cell with the direction reversed, which is the reference swap algorithm's
// border rule (atomicBlock/blockLattice3D.hh:403-427).  Periodic axes wrap,
// which is what the periodic envelopes of MultiBlockLattice3D amount to
// (multiBlock/multiBlockLattice3D.hh:253-357).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>

#include "d3q19.cuh"

namespace plbgpu {

// Loads of the 2-byte storage forms carry the L2::256B prefetch-size hint: a
// warp's 16- or 32-bit accesses cover 64-128 bytes of a plane, and the hint
// lets the L2 fetch the 256-byte segment the neighbouring warps read next
// (+1.8-1.9% for BF16 and FP16 storage on the channel past a sphere; same
// values loaded).
__device__ __forceinline__ unsigned ldPair256(const void* p) {
    unsigned u;
    asm volatile("ld.global.L2::256B.b32 %0, [%1];" : "=r"(u) : "l"(p));
    return u;
}
__device__ __forceinline__ unsigned short ldOne256(const void* p) {
    unsigned short u;
    asm volatile("ld.global.L2::256B.b16 %0, [%1];" : "=h"(u) : "l"(p));
    return u;
}
template <typename S> struct StoreT;
// Every storage type has a store with a `salt` argument; only the
// stochastically rounded BF16 type uses it.
template <> struct StoreT<double> {
    using R = double; using F = double;
    static __device__ __forceinline__ double ld(const double* p) { return *p; }
    static __device__ __forceinline__ void st(double* p, double v) { *p = v; }
    static __device__ __forceinline__ void st(double* p, double v, unsigned) { *p = v; }
};
template <> struct StoreT<float> {
    using R = float; using F = float;
    static __device__ __forceinline__ float ld(const float* p) { return *p; }
    static __device__ __forceinline__ void st(float* p, float v) { *p = v; }
    static __device__ __forceinline__ void st(float* p, float v, unsigned) { *p = v; }
};
template <> struct StoreT<__nv_bfloat16> {
    using R = float; using F = float;
    static __device__ __forceinline__ float ld(const __nv_bfloat16* p) {
        return __uint_as_float((unsigned)ldOne256(p) << 16);
    }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }
    // two adjacent values; p is 4-byte aligned
    static __device__ __forceinline__ void ld2(const __nv_bfloat16* p, float& a, float& b) {
        const unsigned u = ldPair256(p);   // low half: p[0]
        float2 v = make_float2(__uint_as_float(u << 16), __uint_as_float(u & 0xffff0000u));
        a = v.x; b = v.y;
    }
    static __device__ __forceinline__ void st2(__nv_bfloat16* p, float a, float b) {
        *reinterpret_cast<__nv_bfloat162*>(p) = __floats2bfloat162_rn(a, b);
    }
    static __device__ __forceinline__ void st(__nv_bfloat16* p, float v, unsigned) { st(p, v); }
    static __device__ __forceinline__ void st2(__nv_bfloat16* p, float a, float b, unsigned) { st2(p, a, b); }
};
template <> struct StoreT<__half> {
    using R = float; using F = float;
    static __device__ __forceinline__ float ld(const __half* p) {
        return __half2float(__ushort_as_half(ldOne256(p)));
    }
    static __device__ __forceinline__ void st(__half* p, float v) { *p = __float2half_rn(v); }
    static __device__ __forceinline__ void ld2(const __half* p, float& a, float& b) {
        const unsigned u = ldPair256(p);   // low half: p[0]
        float2 v = make_float2(__half2float(__ushort_as_half((unsigned short)(u & 0xffffu))),
                               __half2float(__ushort_as_half((unsigned short)(u >> 16))));
        a = v.x; b = v.y;
    }
    static __device__ __forceinline__ void st2(__half* p, float a, float b) {
        *reinterpret_cast<__half2*>(p) = __floats2half2_rn(a, b);
    }
    static __device__ __forceinline__ void st(__half* p, float v, unsigned) { st(p, v); }
    static __device__ __forceinline__ void st2(__half* p, float a, float b, unsigned) { st2(p, a, b); }
};

// BF16 storage written with stochastic rounding: the 16 bits dropped from the
// FP32 value are compared with 16 pseudo-random bits, so a value rounds up
// with probability equal to its distance from the lower BF16 neighbour and
// the rounding error has zero mean.  Round-to-nearest makes the error of the
// stored populations a deterministic function of the state, which biases the
// conserved moments the same way step after step.  The random bits come from
// a short multiplicative integer hash of the slot address and a per-step
// salt (high half of the product after an xorshift), so a run is
// reproducible.
struct bf16sr {
    __nv_bfloat16 v;
};

__device__ __forceinline__ unsigned srBits(const void* p, unsigned salt) {
    unsigned h = ((unsigned)(reinterpret_cast<unsigned long long>(p) >> 1) ^ salt) * 0x9E3779B1u;
    h ^= h >> 15;
    return h * 0x85EBCA77u;
}

// FP32 -> BF16 rounding up when the dropped 16 bits plus 16 random bits carry.
__device__ __forceinline__ unsigned short bf16Stochastic(float v, unsigned bits) {
    unsigned u = __float_as_uint(v);
    u += bits >> 16;
    return (unsigned short)(u >> 16);
}

template <> struct StoreT<bf16sr> {
    using R = float; using F = float;
    static __device__ __forceinline__ float ld(const bf16sr* p) { return __bfloat162float(p->v); }
    static __device__ __forceinline__ void st(bf16sr* p, float v, unsigned salt) {
        *reinterpret_cast<unsigned short*>(p) = bf16Stochastic(v, srBits(p, salt));
    }
    static __device__ __forceinline__ void st(bf16sr* p, float v) { st(p, v, 0u); }
    static __device__ __forceinline__ void ld2(const bf16sr* p, float& a, float& b) {
        const unsigned u = ldPair256(p);   // low half: p[0]
        float2 v = make_float2(__uint_as_float(u << 16), __uint_as_float(u & 0xffff0000u));
        a = v.x; b = v.y;
    }
    static __device__ __forceinline__ void st2(bf16sr* p, float a, float b, unsigned salt) {
        const unsigned h = srBits(p, salt);
        const unsigned lo = bf16Stochastic(a, h), hi = bf16Stochastic(b, h << 16);
        *reinterpret_cast<unsigned*>(p) = lo | (hi << 16);
    }
    static __device__ __forceinline__ void st2(bf16sr* p, float a, float b) { st2(p, a, b, 0u); }
};

struct DevLattice {
    void* pop;              // 19 planes of `stride` elements of the storage type
    long long stride;       // elements per plane (>= n, padded)
    const uint8_t* flags;   // n
    const uint32_t* mebb;   // n, fluid-direction masks of momentum-exchange cells (or null)
    const double* bc;       // 3 planes of n: face velocity / density (or null)
    const void* force;      // 3 planes of n: Guo force in F (or null)
    const void* ext;        // 4 planes of n in F: external rho-bar, jx, jy, jz (or null)
    int sparse;             // some cells are K_NONE (outside every kept block)
    int nx, ny, nz;
    int per[3];
    long long n;
    unsigned* status;       // device error word (kStatusNonFinite)
    int xRow0, xRows;       // interior rows stepped: 1 + xRow0 <= x <= xRow0 + xRows (0 and nx - 2 for
                            // a whole step; an x-slab of the domain for plbgpu_run_host)
    int rowFacesDone;       // the face cells of interior rows were completed before this launch
                            // (completeFaceListKernel): the interior-row kernels skip their completion
    int rowForm;            // interior-row kernel: 0 the default (two cells per thread for the 2-byte
                            // forms), 1 one cell per thread (every form), 2 / 4 four / eight cells per
                            // thread with 64- / 128-bit vectors (2-byte forms, rows of 8k cells), 3 two
                            // cells per thread with packed 32-bit words (2-byte forms, rows of 2k cells)
    // Sparse domains: tiles (x, y, z0, z1) of at most kTileCells cells of a
    // row.  Dense tiles -- the 3x3 rows around them hold no cell outside the
    // lattice from z0 - 1 to z1 -- take the interior-row kernels; the other
    // tiles with live cells take the general kernel (null: no lists, every
    // row general).
    const int4* denseTiles;
    int nDense;
    const int4* generalTiles;
    int nGeneral;
    // Interior-row tiles next to dropped blocks: the one-cell row kernel with
    // a per-cell mask of the neighbours outside the lattice (tileMasks, one
    // 32-bit word per cell, kTileCells per tile).
    const int4* maskedTiles;
    int nMasked;
    const uint32_t* tileMasks;
};

// Cells of a row tile of a sparse domain's step lists; the kernels run several
// tiles per block (blockDim / threads per tile).
constexpr int kTileCells = 32;

// Bits of DevLattice::status.  A statistics step that meets a NaN or an
// infinity in the density or kinetic-energy sums of a block (a population of
// one of its cells is not finite: the run has diverged) sets kStatusNonFinite;
// the host reports it as PLBGPU_ERR_STATE at the next synchronization.
constexpr unsigned kStatusNonFinite = 1u;

template <typename R>
struct StepParams {
    BgkConst<R> bgk;
    R invRho0;      // incompressible BGK 1/rho0
    int pending;    // boundary faces still need their post-stream completion
    unsigned seed;  // per-step salt of the stochastically rounded storage
    int external;   // collide with rho-bar and j from L.ext (collideExternal)
};

struct StatsAcc {
    double sumRhoBar;
    double sumUSqr;
    unsigned long long count;
    unsigned long long maxBits;   // bit pattern of the max (non-negative doubles order as integers)
    double drag[3];
    double pad;
};

// The statistics are accumulated into kStatsSlots copies of StatsAcc, one per
// block index modulo kStatsSlots, and summed on the host: atomics from
// thousands of blocks on one address would serialize the whole step.
constexpr int kStatsSlots = 64;

__device__ __forceinline__ StatsAcc* statsSlot(StatsAcc* acc) {
    const unsigned b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    return acc + (b & (kStatsSlots - 1));
}

struct ReduceAcc {
    double sumEnergy;   // sum |u|^2
    double sumRhoBar;
    unsigned long long cells;   // cells of the lattice in the box
};

// Offsets along one axis for a move of -1 / +1, or "invalid" outside a
// non-periodic domain.
struct AxisMoves {
    long long offM, offP;
    bool okM, okP;
};

__device__ __forceinline__ AxisMoves axisMoves(int p, int n, int per, long long stride) {
    AxisMoves a;
    a.okM = (p > 0) || per;
    a.okP = (p < n - 1) || per;
    a.offM = (p > 0) ? -stride : (long long)(n - 1) * stride;
    a.offP = (p < n - 1) ? stride : -(long long)(n - 1) * stride;
    return a;
}

struct Neighbourhood {
    AxisMoves ax, ay, az;
    // Move by s * c_i; returns false when leaving a non-periodic domain.
    __device__ __forceinline__ bool move(int i, int s, long long& off) const {
        int cx = s * cdir(i, 0), cy = s * cdir(i, 1), cz = s * cdir(i, 2);
        bool ok = true;
        off = 0;
        if (cx < 0) { ok &= ax.okM; off += ax.offM; } else if (cx > 0) { ok &= ax.okP; off += ax.offP; }
        if (cy < 0) { ok &= ay.okM; off += ay.offM; } else if (cy > 0) { ok &= ay.okP; off += ay.offP; }
        if (cz < 0) { ok &= az.okM; off += az.offM; } else if (cz > 0) { ok &= az.okP; off += az.offP; }
        return ok;
    }
};

__device__ __forceinline__ Neighbourhood neighbourhood(const DevLattice& L, int x, int y, int z) {
    Neighbourhood nb;
    nb.ax = axisMoves(x, L.nx, L.per[0], (long long)L.ny * L.nz);
    nb.ay = axisMoves(y, L.ny, L.per[1], (long long)L.nz);
    nb.az = axisMoves(z, L.nz, L.per[2], 1);
    return nb;
}

// The streaming move of cell idx: on a sparse domain a neighbour outside the
// lattice counts like the outside of the domain (the domain-edge rule).
// SPARSE = false compiles the check out (the step kernels of dense domains).
template <bool SPARSE = true>
__device__ __forceinline__ bool liveMove(const DevLattice& L, const Neighbourhood& nb, long long idx, int i, int s,
                                         long long& off) {
    bool ok = nb.move(i, s, off);
    if constexpr (SPARSE) {
        if (L.sparse && ok) ok = L.flags[idx + off] != K_NONE;
    }
    return ok;
}

// Read the 19 post-stream populations of cell idx for the given parity.
template <typename S, bool ODD, bool SPARSE = true>
__device__ __forceinline__ void loadCell(const DevLattice& L, const Neighbourhood& nb, long long idx,
                                         typename StoreT<S>::R* f) {
    const S* P = static_cast<const S*>(L.pop);
    const long long st = L.stride;
    f[0] = StoreT<S>::ld(P + idx);
#pragma unroll
    for (int i = 1; i < 19; ++i) {
        if (!ODD) {
            f[i] = StoreT<S>::ld(P + i * st + idx);
        } else {
            long long off;
            bool ok = liveMove<SPARSE>(L, nb, idx, i, -1, off);
            f[i] = ok ? StoreT<S>::ld(P + opp(i) * st + idx + off) : StoreT<S>::ld(P + i * st + idx);
        }
    }
}

// Write the 19 post-collision populations of cell idx for the given parity.
template <typename S, bool ODD, bool SPARSE = true>
__device__ __forceinline__ void storeCell(const DevLattice& L, const Neighbourhood& nb, long long idx,
                                          const typename StoreT<S>::R* f, unsigned salt) {
    S* P = static_cast<S*>(L.pop);
    const long long st = L.stride;
    StoreT<S>::st(P + idx, f[0], salt);
#pragma unroll
    for (int i = 1; i < 19; ++i) {
        if (!ODD) {
            StoreT<S>::st(P + opp(i) * st + idx, f[i], salt);
        } else {
            long long off;
            bool ok = liveMove<SPARSE>(L, nb, idx, i, +1, off);
            if (ok) StoreT<S>::st(P + i * st + idx + off, f[i], salt);
            else StoreT<S>::st(P + opp(i) * st + idx, f[i], salt);
        }
    }
}

// Where f_i(x) of the post-stream state lives for the given parity (used by
// the transfer kernels, which read and write the state in place).
template <bool ODD>
__device__ __forceinline__ long long slotOf(const DevLattice& L, const Neighbourhood& nb, long long idx, int i) {
    if (!ODD || i == 0) return (long long)i * L.stride + idx;
    long long off;
    bool ok = liveMove(L, nb, idx, i, -1, off);
    return ok ? (long long)opp(i) * L.stride + idx + off : (long long)i * L.stride + idx;
}

template <typename R>
__device__ __forceinline__ void swapHalves(R* f) {
#pragma unroll
    for (int i = 1; i <= 9; ++i) {
        R t = f[i]; f[i] = f[i + 9]; f[i + 9] = t;
    }
}

template <typename R>
__device__ __forceinline__ void completeIfFace(const DevLattice& L, long long idx, int k, R* f) {
    double v[3] = {L.bc[idx], L.bc[L.n + idx], L.bc[2 * L.n + idx]};
    R tmp[19];
#pragma unroll
    for (int i = 0; i < 19; ++i) tmp[i] = f[i];
    completeFace<R>(tmp, k, v);
#pragma unroll
    for (int i = 0; i < 19; ++i) f[i] = tmp[i];
}

__device__ __forceinline__ double warpSum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ unsigned long long warpSumU(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ unsigned long long warpMaxU(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_down_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// One cell's collision; returns true when the cell gathers statistics.  EXT:
// the external rho-bar / j form (a compile-time variant, so that the plain
// step carries none of its code).
template <typename S, bool EXT>
__device__ __forceinline__ bool collideCell(const DevLattice& L, const StepParams<typename StoreT<S>::R>& P,
                                            long long idx, int k, typename StoreT<S>::R* f,
                                            typename StoreT<S>::R& rhoBar, typename StoreT<S>::R& uSqr,
                                            StatsAcc* acc, bool stats) {
    using R = typename StoreT<S>::R;
    using F = typename StoreT<S>::F;
    R j[3];
    if constexpr (EXT) {
        // ExternalRhoJcollideAndStream3D (dynamicsProcessor3D.hh:41-56):
        // Dynamics::collideExternal with the fields' rho-bar and j.  BGK (and
        // the BGK base of boundary cells) and IncBGK collide on the given
        // moments and gather no statistics (isoThermalDynamics.hh:333-338,
        // 1422-1427); Guo-forced BGK shifts every population by the change of
        // equilibrium, then collides as usual (core/dynamics.hh:131-145);
        // bounce-back, momentum exchange and no-dynamics are unchanged.
        const F* e = static_cast<const F*>(L.ext);
        const R rbE = (R)e[idx];
        const R jE[3] = {(R)e[L.n + idx], (R)e[2 * L.n + idx], (R)e[3 * L.n + idx]};
        if (bgkBase(k) || k == K_INCBGK) {
            uSqr = bgkCollide<R>(f, rbE, jE, P.bgk, k == K_INCBGK ? P.invRho0 : invRhoOf(rbE));
            rhoBar = rbE;
            return false;
        }
        if (k == K_GUO) {
            R oldRb, oldJ[3];
            rhoBarJ<R>(f, oldRb, oldJ);
            const R oldJsqr = oldJ[0] * oldJ[0] + oldJ[1] * oldJ[1] + oldJ[2] * oldJ[2];
            const R jSqr = jE[0] * jE[0] + jE[1] * jE[1] + jE[2] * jE[2];
            const R oldInv = invRhoOf(oldRb), newInv = invRhoOf(rbE);
#pragma unroll
            for (int i = 0; i < 19; ++i) {
                const R oldEq = bgkEq<R>(i, oldRb, oldInv, oldJ, oldJsqr);
                const R newEq = bgkEq<R>(i, rbE, newInv, jE, jSqr);
                f[i] += newEq - oldEq;
            }
        }
    }
    if (bgkBase(k)) {
        // isoThermalDynamics.hh:319-330; faces, edges and corners use their
        // BGK base collide.
        rhoBarJ<R>(f, rhoBar, j);
        uSqr = bgkCollide<R>(f, rhoBar, j, P.bgk, invRhoOf(rhoBar));
        return true;
    }
    switch (k) {
    case K_GUO: {  // externalForceDynamics.hh:215-234
        const F* fp = static_cast<const F*>(L.force);
        R Fv[3] = {(R)fp[idx], (R)fp[L.n + idx], (R)fp[2 * L.n + idx]};
        R rb = rhoBarSeq<R>(f);
        R rb2, jj[3], u[3];
        rhoBarJ<R>(f, rb2, jj);
        R invRho = invRhoOf(rb2);
#pragma unroll
        for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho + Fv[d] / (R)2;
        R rho = rb + (R)1;
#pragma unroll
        for (int d = 0; d < 3; ++d) j[d] = rho * u[d];
        uSqr = bgkCollide<R>(f, rb, j, P.bgk, invRhoOf(rb));
        addGuoForce<R>(f, Fv, u, P.bgk.omega);
        rhoBar = rb;
        return true;
    }
    case K_INCBGK:  // isoThermalDynamics.hh:1408-1419
        rhoBarJ<R>(f, rhoBar, j);
        uSqr = bgkCollide<R>(f, rhoBar, j, P.bgk, P.invRho0);
        return true;
    case K_BB:  // core/dynamics.hh:783-790
        swapHalves(f);
        return false;
    case K_MEBB: {  // bounceBackModels.hh:100-136
        if (stats) {
            uint32_t mask = L.mebb[idx];
            double mom[3] = {0., 0., 0.};
#pragma unroll
            for (int i = 1; i < 19; ++i) {
                if (!(mask & (1u << i))) continue;
                double fo = (double)f[opp(i)];
                if (cdir(i, 0)) mom[0] += (double)2 * cdir(i, 0) * fo;
                if (cdir(i, 1)) mom[1] += (double)2 * cdir(i, 1) * fo;
                if (cdir(i, 2)) mom[2] += (double)2 * cdir(i, 2) * fo;
            }
            StatsAcc* a = statsSlot(acc);
            atomicAdd(&a->drag[0], -mom[0]);
            atomicAdd(&a->drag[1], -mom[1]);
            atomicAdd(&a->drag[2], -mom[2]);
        }
        swapHalves(f);
        return false;
    }
    default:  // K_NODYN, K_NONE
        return false;
    }
}

// Block-wide sum of the per-thread statistics, one set of atomics per block
// on the block's slot.  Every thread of the block must call it.
__device__ __forceinline__ void flushStats(double sR, double sU, unsigned long long cnt, unsigned long long mx,
                                           StatsAcc* acc, unsigned* status) {
    __shared__ double shR[32], shU[32];
    __shared__ unsigned long long shC[32], shM[32];
    sR = warpSum(sR);
    sU = warpSum(sU);
    cnt = warpSumU(cnt);
    mx = warpMaxU(mx);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
        shR[w] = sR;
        shU[w] = sU;
        shC[w] = cnt;
        shM[w] = mx;
    }
    __syncthreads();
    if (w == 0) {
        sR = lane < nw ? shR[lane] : 0.;
        sU = lane < nw ? shU[lane] : 0.;
        cnt = lane < nw ? shC[lane] : 0ull;
        mx = lane < nw ? shM[lane] : 0ull;
        sR = warpSum(sR);
        sU = warpSum(sU);
        cnt = warpSumU(cnt);
        mx = warpMaxU(mx);
        if (lane == 0 && cnt > 0) {
            // one test per block: a NaN or infinity of any cell reaches the sums
            if (!isfinite(sR) || !isfinite(sU)) atomicOr(status, kStatusNonFinite);
            StatsAcc* a = statsSlot(acc);
            atomicAdd(&a->sumRhoBar, sR);
            atomicAdd(&a->sumUSqr, sU);
            atomicAdd(&a->count, cnt);
            atomicMax(&a->maxBits, mx);
        }
    }
}

template <bool STATS>
__device__ __forceinline__ void accumulateStats(bool gathers, double rhoBar, double uSqr, StatsAcc* acc,
                                                unsigned* status) {
    if (!STATS) return;
    flushStats(gathers ? rhoBar : 0., gathers ? uSqr : 0., gathers ? 1ull : 0ull,
               gathers ? (unsigned long long)__double_as_longlong(uSqr) : 0ull, acc, status);
}

// General cell update: any position, periodic wrap and the domain-edge rule.
template <typename S, bool ODD, bool STATS, bool EXT, bool SPARSE>
__device__ __forceinline__ bool processCellGeneral(const DevLattice& L, const StepParams<typename StoreT<S>::R>& P,
                                                   int x, int y, int z, StatsAcc* acc,
                                                   typename StoreT<S>::R& rhoBar, typename StoreT<S>::R& uSqr) {
    using R = typename StoreT<S>::R;
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    const int k = L.flags[idx];
    if (k == K_NONE) return false;
    Neighbourhood nb = neighbourhood(L, x, y, z);
    R f[19];
    loadCell<S, ODD, SPARSE>(L, nb, idx, f);
    if (P.pending && isFace(k)) completeIfFace<R>(L, idx, k, f);
    bool g = collideCell<S, EXT>(L, P, idx, k, f, rhoBar, uSqr, acc, STATS);
    storeCell<S, ODD, SPARSE>(L, nb, idx, f, P.seed);
    return g;
}

// Population planes and the neighbour offsets c_i . (ny*nz, nz, 1) passed by
// value (kernel parameters live in the constant bank).
template <typename S>
struct Planes {
    S* p[19];
};
struct Deltas {
    int d[19];
};

// Cells of a row with 1 <= x <= nx-2 and 1 <= y <= ny-2: a neighbour can only
// leave the domain (or wrap) along z, so every population address is
// plane_i + idx +- delta_i with uniform deltas and a 32-bit cell index; only
// the ten populations that move along z carry a per-thread wrap / reflection
// select.
template <typename S, bool ODD, bool MASKED = false>
struct RowCell {
    int idx, wrapM, wrapP;
    bool okM, okP;
    // MASKED: bit k set when the neighbour x + c_k is outside the lattice (a
    // sparse domain's dropped block): that population follows the
    // domain-edge rule, like one leaving a non-periodic box
    unsigned gone = 0;

    __device__ __forceinline__ RowCell(const DevLattice& L, int x, int y, int z) {
        idx = (x * L.ny + y) * L.nz + z;
        const bool zlo = (z == 0), zhi = (z == L.nz - 1);
        wrapM = zlo ? L.nz : 0;    // a -1 move along z at z = 0 wraps to nz-1
        wrapP = zhi ? -L.nz : 0;   // a +1 move along z at z = nz-1 wraps to 0
        okM = !zlo || L.per[2];
        okP = !zhi || L.per[2];
    }

    __device__ __forceinline__ void load(const Planes<S>& Pl, const Deltas& D, typename StoreT<S>::R* f) const {
        f[0] = StoreT<S>::ld(Pl.p[0] + idx);
#pragma unroll
        for (int i = 1; i < 19; ++i) {
            if (!ODD) {
                f[i] = StoreT<S>::ld(Pl.p[i] + idx);
            } else {
                const int mz = -cdir(i, 2);   // the source is x - c_i = x + c_opp(i)
                if (mz == 0 && !MASKED) {
                    f[i] = StoreT<S>::ld(Pl.p[opp(i)] + (idx - D.d[i]));
                } else {
                    bool ok = mz == 0 ? true : (mz < 0 ? okM : okP);
                    if (MASKED) ok = ok && !((gone >> opp(i)) & 1u);
                    const int off = -D.d[i] + (mz == 0 ? 0 : (mz < 0 ? wrapM : wrapP));
                    const S* a = ok ? Pl.p[opp(i)] + (idx + off) : Pl.p[i] + idx;
                    f[i] = StoreT<S>::ld(a);
                }
            }
        }
    }

    __device__ __forceinline__ void store(const Planes<S>& Pl, const Deltas& D, const typename StoreT<S>::R* f,
                                          unsigned salt) const {
        StoreT<S>::st(Pl.p[0] + idx, f[0], salt);
#pragma unroll
        for (int i = 1; i < 19; ++i) {
            if (!ODD) {
                StoreT<S>::st(Pl.p[opp(i)] + idx, f[i], salt);
            } else {
                const int cz = cdir(i, 2);    // the destination is x + c_i
                if (cz == 0 && !MASKED) {
                    StoreT<S>::st(Pl.p[i] + (idx + D.d[i]), f[i], salt);
                } else {
                    bool ok = cz == 0 ? true : (cz < 0 ? okM : okP);
                    if (MASKED) ok = ok && !((gone >> i) & 1u);
                    const int off = D.d[i] + (cz == 0 ? 0 : (cz < 0 ? wrapM : wrapP));
                    S* a = ok ? Pl.p[i] + (idx + off) : Pl.p[opp(i)] + idx;
                    StoreT<S>::st(a, f[i], salt);
                }
            }
        }
    }
};

// Cells per thread of the row kernel and its residency target (blocks of 128
// threads per SM).
template <typename S> struct RowShape { static constexpr int cells = 1, blocks = 8; };
template <> struct RowShape<double> { static constexpr int cells = 1, blocks = 5; };

// Rows with 1 <= x <= nx-2 and 1 <= y <= ny-2 (all z): nearly all of the time
// step.  A block covers RowShape::cells * blockDim.x consecutive cells of one
// row; thread t owns cells t, t + blockDim.x, ... (coalesced planes).
template <typename S, bool ODD, bool STATS, bool EXT, bool MASKED = false>
__global__ void __launch_bounds__(128, RowShape<S>::blocks)
    rowStepKernel(DevLattice L, Planes<S> Pl, Deltas D, StepParams<typename StoreT<S>::R> P, StatsAcc* acc) {
    using R = typename StoreT<S>::R;
    constexpr int NC = RowShape<S>::cells;
    static_assert(!MASKED || NC == 1, "masked tiles: one cell per thread");
    int x = blockIdx.z + 1 + L.xRow0, y = blockIdx.y + 1;
    int z0 = blockIdx.x * blockDim.x * NC + threadIdx.x, zEnd = L.nz;
    unsigned gone = 0;
    const int4* tiles = MASKED ? L.maskedTiles : L.denseTiles;
    if (tiles) {          // blockDim / kTileCells tiles per block (NC = 1)
        const int r = (blockIdx.y + gridDim.y * blockIdx.z) * (blockDim.x / kTileCells) + threadIdx.x / kTileCells;
        zEnd = -1;        // no cells past the list's end
        if (r < (MASKED ? L.nMasked : L.nDense)) {
            const int4 t = tiles[r];
            x = t.x;
            y = t.y;
            z0 = t.z + threadIdx.x % kTileCells;
            zEnd = t.w;
            if (MASKED) gone = L.tileMasks[(long long)r * kTileCells + threadIdx.x % kTileCells];
        }
    }
    R f[NC][19];
    int kind[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const int z = z0 + c * blockDim.x;
        kind[c] = K_NONE;
        if (z < zEnd) {
            RowCell<S, ODD, MASKED> rc(L, x, y, z);
            rc.gone = gone;
            kind[c] = L.flags[rc.idx];
            if (kind[c] != K_NONE) rc.load(Pl, D, f[c]);
        }
    }
    double sR = 0., sU = 0.;
    unsigned long long cnt = 0, mx = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        if (kind[c] == K_NONE) continue;
        RowCell<S, ODD, MASKED> rc(L, x, y, z0 + c * blockDim.x);
        rc.gone = gone;
        R rhoBar = R(0), uSqr = R(0);
        if (P.pending && !L.rowFacesDone && isFace(kind[c])) completeIfFace<R>(L, rc.idx, kind[c], f[c]);
        bool g = collideCell<S, EXT>(L, P, rc.idx, kind[c], f[c], rhoBar, uSqr, acc, STATS);
        rc.store(Pl, D, f[c], P.seed);
        if (STATS && g) {
            sR += (double)rhoBar;
            sU += (double)uSqr;
            cnt += 1;
            unsigned long long b = (unsigned long long)__double_as_longlong((double)uSqr);
            mx = b > mx ? b : mx;
        }
    }
    if (STATS) flushStats(sR, sU, cnt, mx, acc, L.status);
}

// ---------------------------------------------------------------- paired row kernel
//
// 2-byte storage forms: each thread owns two adjacent cells (z even, z + 1).
// Populations that stay in the same z column (c_z = 0) move as one aligned
// 32-bit word for both cells -- every population in the even step, nine of
// nineteen in the odd step -- halving the memory instructions and doubling
// the bytes per request; the other ten go as 16-bit values with the row-end
// wrap / reflection selects of RowCell.  Needs nz even (rows and planes start
// on 4-byte boundaries).
template <typename S, bool ODD, bool STATS, bool EXT>
__global__ void __launch_bounds__(128, 8)
    pairRowStepKernel(DevLattice L, Planes<S> Pl, Deltas D, StepParams<typename StoreT<S>::R> P, StatsAcc* acc) {
    using R = typename StoreT<S>::R;
    int x = blockIdx.z + 1 + L.xRow0, y = blockIdx.y + 1;
    int zA = 2 * (blockIdx.x * blockDim.x + threadIdx.x), zEnd = L.nz;
    if (L.denseTiles) {   // blockDim / (kTileCells / 2) tiles per block
        constexpr int TT = kTileCells / 2;
        const int r = (blockIdx.y + gridDim.y * blockIdx.z) * (blockDim.x / TT) + threadIdx.x / TT;
        zEnd = -1;        // no cells past the list's end
        if (r < L.nDense) {
            const int4 t = L.denseTiles[r];
            x = t.x;
            y = t.y;
            zA = t.z + 2 * (threadIdx.x % TT);
            zEnd = t.w;
        }
    }
    double sR = 0., sU = 0.;
    unsigned long long cnt = 0, mx = 0;
    if (zA < zEnd) {
        RowCell<S, ODD> ca(L, x, y, zA), cb(L, x, y, zA + 1);
        const int kA = L.flags[ca.idx], kB = L.flags[cb.idx];
        R fa[19], fb[19];
        StoreT<S>::ld2(Pl.p[0] + ca.idx, fa[0], fb[0]);
#pragma unroll
        for (int i = 1; i < 19; ++i) {
            if (!ODD) {
                StoreT<S>::ld2(Pl.p[i] + ca.idx, fa[i], fb[i]);
            } else if (cdir(i, 2) == 0) {
                StoreT<S>::ld2(Pl.p[opp(i)] + (ca.idx - D.d[i]), fa[i], fb[i]);
            } else {
                const int mz = -cdir(i, 2);
                {
                    const bool ok = mz < 0 ? ca.okM : ca.okP;
                    const int off = -D.d[i] + (mz < 0 ? ca.wrapM : ca.wrapP);
                    fa[i] = StoreT<S>::ld(ok ? Pl.p[opp(i)] + (ca.idx + off) : Pl.p[i] + ca.idx);
                }
                {
                    const bool ok = mz < 0 ? cb.okM : cb.okP;
                    const int off = -D.d[i] + (mz < 0 ? cb.wrapM : cb.wrapP);
                    fb[i] = StoreT<S>::ld(ok ? Pl.p[opp(i)] + (cb.idx + off) : Pl.p[i] + cb.idx);
                }
            }
        }
        const bool liveA = kA != K_NONE, liveB = kB != K_NONE;
        R rbA = R(0), usA = R(0), rbB = R(0), usB = R(0);
        bool gA = false, gB = false;
        if (liveA) {
            if (P.pending && !L.rowFacesDone && isFace(kA)) completeIfFace<R>(L, ca.idx, kA, fa);
            gA = collideCell<S, EXT>(L, P, ca.idx, kA, fa, rbA, usA, acc, STATS);
        }
        if (liveB) {
            if (P.pending && !L.rowFacesDone && isFace(kB)) completeIfFace<R>(L, cb.idx, kB, fb);
            gB = collideCell<S, EXT>(L, P, cb.idx, kB, fb, rbB, usB, acc, STATS);
        }
        if (liveA && liveB) {
            StoreT<S>::st2(Pl.p[0] + ca.idx, fa[0], fb[0], P.seed);
#pragma unroll
            for (int i = 1; i < 19; ++i) {
                if (!ODD) {
                    StoreT<S>::st2(Pl.p[opp(i)] + ca.idx, fa[i], fb[i], P.seed);
                } else if (cdir(i, 2) == 0) {
                    StoreT<S>::st2(Pl.p[i] + (ca.idx + D.d[i]), fa[i], fb[i], P.seed);
                } else {
                    const int cz = cdir(i, 2);
                    {
                        const bool ok = cz < 0 ? ca.okM : ca.okP;
                        const int off = D.d[i] + (cz < 0 ? ca.wrapM : ca.wrapP);
                        StoreT<S>::st(ok ? Pl.p[i] + (ca.idx + off) : Pl.p[opp(i)] + ca.idx, fa[i], P.seed);
                    }
                    {
                        const bool ok = cz < 0 ? cb.okM : cb.okP;
                        const int off = D.d[i] + (cz < 0 ? cb.wrapM : cb.wrapP);
                        StoreT<S>::st(ok ? Pl.p[i] + (cb.idx + off) : Pl.p[opp(i)] + cb.idx, fb[i], P.seed);
                    }
                }
            }
        } else {
            if (liveA) ca.store(Pl, D, fa, P.seed);
            if (liveB) cb.store(Pl, D, fb, P.seed);
        }
        if (STATS) {
            if (gA) {
                sR += (double)rbA; sU += (double)usA; cnt += 1;
                mx = (unsigned long long)__double_as_longlong((double)usA);
            }
            if (gB) {
                sR += (double)rbB; sU += (double)usB; cnt += 1;
                unsigned long long b = (unsigned long long)__double_as_longlong((double)usB);
                mx = b > mx ? b : mx;
            }
        }
    }
    if (STATS) flushStats(sR, sU, cnt, mx, acc, L.status);
}

// Rows on the x or y border of the domain, with the general addressing
// (periodic wrap and the domain-edge rule on every axis).  Row
// blockIdx.y + gridDim.y * blockIdx.z enumerates the border rows: x = 0,
// x = nx-1 (all y), then y = 0, y = ny-1 (1 <= x <= nx-2); when nx < 3 or
// ny < 3 every row is a border row; on a sparse domain the blocks are its
// general tiles (or every row when it has no lists).
template <typename S, bool ODD, bool STATS, bool EXT, bool SPARSE>
__global__ void __launch_bounds__(128, sizeof(S) <= 4 ? 6 : 1) edgeRowStepKernel(DevLattice L, StepParams<typename StoreT<S>::R> P,
                                                          StatsAcc* acc, int rows) {
    using R = typename StoreT<S>::R;
    int z = blockIdx.x * blockDim.x + threadIdx.x, zEnd = L.nz;
    int row = blockIdx.y + gridDim.y * blockIdx.z;
    const bool tiles = SPARSE && L.generalTiles;
    if (tiles) row = row * (blockDim.x / kTileCells) + threadIdx.x / kTileCells;   // several tiles per block
    else if (row >= rows) return;   // whole blocks
    const int nx = L.nx, ny = L.ny;
    int x = 0, y = 0;
    if (tiles) {
        zEnd = -1;                  // no cells past the list's end
        if (row < rows) {
            const int4 t = L.generalTiles[row];
            x = t.x;
            y = t.y;
            z = t.z + threadIdx.x % kTileCells;
            zEnd = t.w;
        }
    } else if (SPARSE || nx < 3 || ny < 3) {
        x = row / ny;
        y = row - x * ny;
    } else if (row < ny) {
        x = 0; y = row;
    } else if (row < 2 * ny) {
        x = nx - 1; y = row - ny;
    } else if (row < 2 * ny + (nx - 2)) {
        x = 1 + row - 2 * ny; y = 0;
    } else {
        x = 1 + row - 2 * ny - (nx - 2); y = ny - 1;
    }
    R rhoBar = R(0), uSqr = R(0);
    bool g = false;
    if (z < zEnd) g = processCellGeneral<S, ODD, STATS, EXT, SPARSE>(L, P, x, y, z, acc, rhoBar, uSqr);
    accumulateStats<STATS>(g, (double)rhoBar, (double)uSqr, acc, L.status);
}

// Complete the boundary faces in place (used before a transfer into a state
// whose faces are still pending).
template <typename S, bool ODD>
__global__ void completeFacesKernel(DevLattice L) {
    using R = typename StoreT<S>::R;
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    if (z >= L.nz) return;
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    const int k = L.flags[idx];
    if (!isFace(k)) return;
    Neighbourhood nb = neighbourhood(L, x, y, z);
    S* Pp = static_cast<S*>(L.pop);
    R f[19];
#pragma unroll
    for (int i = 0; i < 19; ++i) f[i] = StoreT<S>::ld(Pp + slotOf<ODD>(L, nb, idx, i));
    completeIfFace<R>(L, idx, k, f);
#pragma unroll
    for (int i = 0; i < 19; ++i) StoreT<S>::st(Pp + slotOf<ODD>(L, nb, idx, i), f[i]);
}

// The face cells of a list (x, y, z, kind), completed in place before a step:
// the interior-row kernels then find them complete.  A face cell inside an
// interior row (a lid or a face plane across the rows) would otherwise make
// its warp run the completion for one lane while the others wait; listed, the
// completions run in full warps.
template <typename S, bool ODD>
__global__ void completeFaceListKernel(DevLattice L, const int4* __restrict__ cells, int count) {
    using R = typename StoreT<S>::R;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int4 c = cells[t];
    const long long idx = ((long long)c.x * L.ny + c.y) * L.nz + c.z;
    Neighbourhood nb = neighbourhood(L, c.x, c.y, c.z);
    S* Pp = static_cast<S*>(L.pop);
    R f[19];
#pragma unroll
    for (int i = 0; i < 19; ++i) f[i] = StoreT<S>::ld(Pp + slotOf<ODD>(L, nb, idx, i));
    completeIfFace<R>(L, idx, c.w, f);
#pragma unroll
    for (int i = 0; i < 19; ++i) StoreT<S>::st(Pp + slotOf<ODD>(L, nb, idx, i), f[i]);
}

struct Box { int x0, x1, y0, y1, z0, z1; };

// Canonical transfer layout: [x][y][z][19] over the box, z fastest, FP64.
// The buffer may be device memory or, over NVLink-C2C, the caller's host
// memory (pinned or pageable), so a block stages its run of up to kXferCells
// cells of one box row in shared memory and reads or writes the run as one
// contiguous, coalesced stretch of 19 * cells doubles; the slots in the
// population planes are then written or read one cell per thread.
constexpr int kXferCells = 128;

// B: the element type of the transfer buffer (double, or float for the
// single-precision co-processor form).
template <typename S, bool ODD, typename B>
__global__ void __launch_bounds__(kXferCells) extractKernel(DevLattice L, Box b, int pending, B* out) {
    using R = typename StoreT<S>::R;
    __shared__ double sh[kXferCells * 19];
    const int bnz = b.z1 - b.z0 + 1, bny = b.y1 - b.y0 + 1;
    const int dz0 = blockIdx.x * kXferCells;
    const int cnt = min(kXferCells, bnz - dz0);
    const int t = threadIdx.x;
    if (t < cnt) {
        const int z = b.z0 + dz0 + t, y = b.y0 + blockIdx.y, x = b.x0 + blockIdx.z;
        const long long idx = ((long long)x * L.ny + y) * L.nz + z;
        const int k = L.flags[idx];
        R f[19];
        if (k == K_NONE) {   // not part of the lattice: reads as zeros
#pragma unroll
            for (int i = 0; i < 19; ++i) f[i] = R(0);
        } else {
            Neighbourhood nb = neighbourhood(L, x, y, z);
            const S* Pp = static_cast<const S*>(L.pop);
#pragma unroll
            for (int i = 0; i < 19; ++i) f[i] = StoreT<S>::ld(Pp + slotOf<ODD>(L, nb, idx, i));
            if (pending && isFace(k)) completeIfFace<R>(L, idx, k, f);
        }
#pragma unroll
        for (int i = 0; i < 19; ++i) sh[t * 19 + i] = (double)f[i];
    }
    __syncthreads();
    const long long o0 = (((long long)blockIdx.z * bny + blockIdx.y) * bnz + dz0) * 19;
    for (int q = t; q < cnt * 19; q += kXferCells) out[o0 + q] = (B)sh[q];
}

template <typename S, bool ODD, typename B>
__global__ void __launch_bounds__(kXferCells) insertKernel(DevLattice L, Box b, const B* in) {
    __shared__ double sh[kXferCells * 19];
    const int bnz = b.z1 - b.z0 + 1, bny = b.y1 - b.y0 + 1;
    const int dz0 = blockIdx.x * kXferCells;
    const int cnt = min(kXferCells, bnz - dz0);
    const int t = threadIdx.x;
    const long long o0 = (((long long)blockIdx.z * bny + blockIdx.y) * bnz + dz0) * 19;
    for (int q = t; q < cnt * 19; q += kXferCells) sh[q] = (double)in[o0 + q];
    __syncthreads();
    if (t >= cnt) return;
    const int z = b.z0 + dz0 + t, y = b.y0 + blockIdx.y, x = b.x0 + blockIdx.z;
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    if (L.flags[idx] == K_NONE) return;
    Neighbourhood nb = neighbourhood(L, x, y, z);
    S* Pp = static_cast<S*>(L.pop);
#pragma unroll
    for (int i = 0; i < 19; ++i)
        StoreT<S>::st(Pp + slotOf<ODD>(L, nb, idx, i), (typename StoreT<S>::R)sh[t * 19 + i]);
}

// Macroscopic values of one cell the way each dynamics reports them
// (Cell::computeVelocity / computeRhoBar / computeDensity), on the
// post-stream, face-completed state.  Returns false for cells outside the
// lattice.  rho is computeDensity, rb is computeRhoBar.
template <typename S, bool ODD>
__device__ __forceinline__ bool cellMacroscopic(const DevLattice& L, int x, int y, int z, int pending,
                                                typename StoreT<S>::R invRho0, double bbRho,
                                                typename StoreT<S>::R* u, typename StoreT<S>::R& rb,
                                                double& rho) {
    using R = typename StoreT<S>::R;
    using F = typename StoreT<S>::F;
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    const int k = L.flags[idx];
    if (k == K_NONE) return false;
    Neighbourhood nb = neighbourhood(L, x, y, z);
    const S* Pp = static_cast<const S*>(L.pop);
    R f[19];
#pragma unroll
    for (int i = 0; i < 19; ++i) f[i] = StoreT<S>::ld(Pp + slotOf<ODD>(L, nb, idx, i));
    if (pending && isFace(k)) completeIfFace<R>(L, idx, k, f);
    u[0] = u[1] = u[2] = R(0);
    rb = R(0);
    if (k == K_BB || k == K_MEBB) {  // core/dynamics.hh:814-829, 875-877
        rb = (R)(bbRho - 1.0);
        rho = bbRho;
        return true;
    }
    if (k == K_NODYN) {  // core/dynamics.hh:994-1008, 1055-1058
        rho = bbRho;
        return true;
    }
    if (k == K_BGK) {  // momentTemplates3D.h:402-408 compute_uLb
        R jj[3], rr;
        rhoBarJ<R>(f, rr, jj);
        rb = rhoBarSeq<R>(f);
        R invRho = invRhoOf(rb);
        for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho;
    } else if (k == K_GUO) {  // externalForceDynamics.hh:58-73
        const F* fp = static_cast<const F*>(L.force);
        R jj[3], rr;
        rhoBarJ<R>(f, rr, jj);
        R invRho = invRhoOf(rr);
        R Fv[3] = {(R)fp[idx], (R)fp[L.n + idx], (R)fp[2 * L.n + idx]};
        for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho + Fv[d] / (R)2;
        rb = rhoBarSeq<R>(f);
    } else if (k == K_INCBGK) {  // isoThermalDynamics.hh:1388-1395
        R jj[3], rr;
        rhoBarJ<R>(f, rr, jj);
        for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho0;
        rb = rhoBarSeq<R>(f);
    } else if (isSurface(k)) {  // StoreVelocityDynamics over BGK: stored u, base density
        for (int d = 0; d < 3; ++d) u[d] = (R)L.bc[d * L.n + idx];
        const R rs = rhoBarSeq<R>(f);
        rho = (double)(rs + (R)1);             // BoundaryCompositeDynamics::computeDensity
        rb = (rs + (R)1) - (R)1;               // StoreVelocityDynamics::computeRhoBar
        return true;
    } else if (isFace(k)) {
        const int fam = faceFamily(k), dir = faceDir(k);
        double v[3] = {L.bc[idx], L.bc[L.n + idx], L.bc[2 * L.n + idx]};
        if (fam == 0 || fam == 2) {  // stored velocity, boundaryDynamics.hh:324-330
            for (int d = 0; d < 3; ++d) u[d] = (R)v[d];
            rb = velFaceRhoBarAny<R>(f, k, (R)v[dir]);
        } else {  // boundaryDynamics.hh:790-812
            rb = (R)v[0] - (R)1;
            pressFaceJAny<R>(f, k, rb, u);
            R invRho = invRhoOf(rb);
            for (int d = 0; d < 3; ++d) { u[d] *= invRho; u[d] += (R)0.5 * (R)0; }
        }
    }
    rho = (double)rb + 1.0;   // fullRho(rhoBar)
    return true;
}

// ---------------------------------------------------------------- edges and corners
//
// External velocity edges and corners of the local regularized condition:
// after the faces, each edge cell, then each corner cell, is rebuilt as
// f_eq(rho, rho u) + fNeq(Pi) from finite differences of its neighbours'
// velocities and densities (OuterVelocityEdgeFunctional3D /
// OuterVelocityCornerFunctional3D, finiteDifferenceBoundaryProcessor3D.hh:
// 141-316).  The host lists the cells (x, y, z, kind) and has checked that
// every neighbour read below lies inside the domain (after the periodic wrap),
// and that an edge reads no edge's or corner's density and a corner no
// corner's density, so that no thread reads populations another one writes.
//
// The processor is written once for any arithmetic type T (the form's R, or
// a dual number of R in the adjoint module) and any population source: a
// source `src(x, y, z, idx, f)` loads the raw post-stream populations of cell
// (x, y, z) = idx into
// f[19].

__device__ __forceinline__ int wrapAxis(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// fullRho(rhoBar) as Cell::computeDensity reports it, rounded to R: the
// density is formed in double ((double)rhoBar + 1) and the finite differences
// use it in R.
template <typename R>
__device__ __forceinline__ R densityOfRhoBar(R rb) { return (R)((double)rb + 1.0); }

// Cell::computeVelocity / computeDensity of a cell of kind k from its raw
// post-stream populations f (completed in place first when the faces are
// pending), the way each dynamics reports them.  rho is the density in R.
template <typename R, typename T>
__device__ __forceinline__ void macroOfPops(const DevLattice& L, long long idx, int k, T* f, int pending, R invRho0,
                                            double bbRho, T* u, T& rho) {
    if (pending && isFace(k)) completeIfFace<T>(L, idx, k, f);
    u[0] = u[1] = u[2] = T(0);
    if (k == K_BB || k == K_MEBB || k == K_NODYN || k == K_NONE) {  // core/dynamics.hh:814-829, 994-1008
        rho = T((R)bbRho);
        return;
    }
    T rb;
    if (k == K_BGK) {  // momentTemplates3D.h:402-408 compute_uLb
        T jj[3], rr;
        rhoBarJ<T>(f, rr, jj);
        rb = rhoBarSeq<T>(f);
        T invRho = invRhoOf(rb);
        for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho;
    } else if (k == K_GUO) {  // externalForceDynamics.hh:58-73
        const R* fp = static_cast<const R*>(L.force);
        T jj[3], rr;
        rhoBarJ<T>(f, rr, jj);
        T invRho = invRhoOf(rr);
        T Fv[3] = {T(fp[idx]), T(fp[L.n + idx]), T(fp[2 * L.n + idx])};
        for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho + Fv[d] / T(2);
        rb = rhoBarSeq<T>(f);
    } else if (k == K_INCBGK) {  // isoThermalDynamics.hh:1388-1395
        T jj[3], rr;
        rhoBarJ<T>(f, rr, jj);
        for (int d = 0; d < 3; ++d) u[d] = jj[d] * T(invRho0);
        rb = rhoBarSeq<T>(f);
    } else if (isSurface(k)) {  // StoreVelocityDynamics over BGK: stored u, base density
        for (int d = 0; d < 3; ++d) u[d] = T((R)L.bc[d * L.n + idx]);
        rho = rhoBarSeq<T>(f) + T(1);        // BoundaryCompositeDynamics::computeDensity
        return;
    } else {  // faces
        const int fam = faceFamily(k), dir = faceDir(k);
        const double v[3] = {L.bc[idx], L.bc[L.n + idx], L.bc[2 * L.n + idx]};
        if (fam == 0 || fam == 2) {  // stored velocity, boundaryDynamics.hh:324-330
            for (int d = 0; d < 3; ++d) u[d] = T((R)v[d]);
            rb = velFaceRhoBarAny<T>(f, k, T((R)v[dir]));
        } else {  // boundaryDynamics.hh:790-812
            rb = T((R)v[0]) - T(1);
            pressFaceJAny<T>(f, k, rb, u);
            T invRho = invRhoOf(rb);
            for (int d = 0; d < 3; ++d) { u[d] *= invRho; u[d] += T(0.5) * T(0); }
        }
    }
    rho = densityOfRhoBar(rb);
}

// Velocity of the cell at p (wrapped): the stored velocity of an edge, a
// corner or a velocity face and the zero of a wall, without reading
// populations (the values macroOfPops gives them), else computeVelocity.
template <typename R, typename T, class Src>
__device__ __forceinline__ void surfaceVelocityAt(const DevLattice& L, const int* p, int pending, R invRho0,
                                                  double bbRho, Src& src, T* u) {
    const int x = wrapAxis(p[0], L.nx), y = wrapAxis(p[1], L.ny), z = wrapAxis(p[2], L.nz);
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    const int k = L.flags[idx];
    if (isSurface(k) || (isFace(k) && (faceFamily(k) == 0 || faceFamily(k) == 2))) {
#pragma unroll
        for (int d = 0; d < 3; ++d) u[d] = T((R)L.bc[d * L.n + idx]);
        return;
    }
    if (k == K_BB || k == K_MEBB || k == K_NODYN || k == K_NONE) {
        u[0] = u[1] = u[2] = T(0);
        return;
    }
    T f[19], rho;
    src(x, y, z, idx, f);
    macroOfPops<R, T>(L, idx, k, f, pending, invRho0, bbRho, u, rho);
}

// Density of the cell at p (wrapped); a wall's without reading populations.
template <typename R, typename T, class Src>
__device__ __forceinline__ T surfaceDensityAt(const DevLattice& L, const int* p, int pending, R invRho0, double bbRho,
                                              Src& src) {
    const int x = wrapAxis(p[0], L.nx), y = wrapAxis(p[1], L.ny), z = wrapAxis(p[2], L.nz);
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    const int k = L.flags[idx];
    if (k == K_BB || k == K_MEBB || k == K_NODYN || k == K_NONE) return T((R)bbRho);
    T f[19], u[3], rho;
    src(x, y, z, idx, f);
    macroOfPops<R, T>(L, idx, k, f, pending, invRho0, bbRho, u, rho);
    return rho;
}

// The finite differences of an edge or corner cell (fd::DirectedGradients3D,
// finiteDifference/finiteDifference3D.h:61-190: first-order one-sided into the
// domain along a normal, d_A u = -normal (u(x - normal e_A) - u(x)); centred
// along an edge, d_A u = (u(x + e_A) - u(x - e_A)) / 2) and its density: the
// mean of the inward neighbours' densities.  g[A][d] = d_A u_d.
template <typename R, typename T, class Src>
__device__ __forceinline__ void surfaceGradients(const DevLattice& L, int4 c, int pending, R invRho0, double bbRho,
                                                 Src& src, T& rho, T (&g)[3][3]) {
    const int p[3] = {c.x, c.y, c.z};
    const long long idx = ((long long)c.x * L.ny + c.y) * L.nz + c.z;
    T vel[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) vel[d] = T((R)L.bc[d * L.n + idx]);
    auto normal = [&](int axis, int nrm) {
        int q[3] = {p[0], p[1], p[2]};
        q[axis] -= nrm;
        T u1[3];
        surfaceVelocityAt<R, T>(L, q, pending, invRho0, bbRho, src, u1);
#pragma unroll
        for (int d = 0; d < 3; ++d) g[axis][d] = T(-nrm) * (-vel[d] + u1[d]);
    };
    if (c.w < K_CORNER) {
        const int e = c.w - K_EDGE, plane = e / 4;
        const int n1 = (e & 2) ? 1 : -1, n2 = (e & 1) ? 1 : -1;
        const int d1 = (plane + 1) % 3, d2 = (plane + 2) % 3;
        int a[3] = {p[0], p[1], p[2]}, b[3] = {p[0], p[1], p[2]};
        a[d1] -= n1;
        b[d2] -= n2;
        const T rho10 = surfaceDensityAt<R, T>(L, a, pending, invRho0, bbRho, src);
        const T rho01 = surfaceDensityAt<R, T>(L, b, pending, invRho0, bbRho, src);
        rho = T(0.5) * (rho01 + rho10);
        int up[3] = {p[0], p[1], p[2]}, um[3] = {p[0], p[1], p[2]};
        up[plane] += 1;
        um[plane] -= 1;
        T uu[3], ud[3];
        surfaceVelocityAt<R, T>(L, up, pending, invRho0, bbRho, src, uu);
        surfaceVelocityAt<R, T>(L, um, pending, invRho0, bbRho, src, ud);
#pragma unroll
        for (int d = 0; d < 3; ++d) g[plane][d] = (uu[d] - ud[d]) / T(2);
        normal(d1, n1);
        normal(d2, n2);
    } else {
        const int q = c.w - K_CORNER;
        const int nrm[3] = {(q & 4) ? 1 : -1, (q & 2) ? 1 : -1, (q & 1) ? 1 : -1};
        T r[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            int nbp[3] = {p[0], p[1], p[2]};
            nbp[a] -= nrm[a];
            r[a] = surfaceDensityAt<R, T>(L, nbp, pending, invRho0, bbRho, src);
        }
        rho = T(1) / T(3) * (r[2] + r[1] + r[0]);
#pragma unroll
        for (int a = 0; a < 3; ++a) normal(a, nrm[a]);
    }
}

// The rebuilt populations from (rho, velocity gradients): off-equilibrium
// stress Pi = -rho / (3 omega) (grad u + grad u^T), then f_eq(rho, rho u) +
// fNeq(Pi) (finiteDifferenceBoundaryProcessor3D.hh:180-206).
template <typename T>
__device__ __forceinline__ void surfaceFromGradients(const T& rho, const T (&g)[3][3], const T* vel, const T& omega,
                                                     T* f) {
    const T sToPi = -rho / T(3) / omega;
    T Pi[6];
    Pi[0] = T(2) * g[0][0] * sToPi;
    Pi[1] = (g[0][1] + g[1][0]) * sToPi;
    Pi[2] = (g[0][2] + g[2][0]) * sToPi;
    Pi[3] = T(2) * g[1][1] * sToPi;
    Pi[4] = (g[1][2] + g[2][1]) * sToPi;
    Pi[5] = T(2) * g[2][2] * sToPi;
    T j[3] = {rho * vel[0], rho * vel[1], rho * vel[2]};
    const T jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    regularizeFromPi<T>(f, rho - T(1), j, jSqr, Pi);
}

// Populations of the AA-ordered state of parity ODD.
template <typename S, bool ODD>
struct AASource {
    const DevLattice& L;
    __device__ __forceinline__ void operator()(int x, int y, int z, long long idx, typename StoreT<S>::R* f) const {
        Neighbourhood nb = neighbourhood(L, x, y, z);
        const S* Pp = static_cast<const S*>(L.pop);
#pragma unroll
        for (int i = 0; i < 19; ++i) f[i] = StoreT<S>::ld(Pp + slotOf<ODD>(L, nb, idx, i));
    }
};

// Gradients and density of one edge or corner cell of the domain's own state,
// as one out-of-line call: the finite differences read up to five
// neighbours, and inlining their macroscopic values into the kernel would
// multiply its code for no gain on a few thousand cells.
template <typename S, bool ODD>
__device__ __noinline__ void surfaceGradientsAA(const DevLattice& L, int4 c, int pending,
                                                typename StoreT<S>::R invRho0, double bbRho,
                                                typename StoreT<S>::R& rho, typename StoreT<S>::R (&g)[3][3]) {
    using R = typename StoreT<S>::R;
    AASource<S, ODD> src{L};
    surfaceGradients<R, R>(L, c, pending, invRho0, bbRho, src, rho, g);
}

// One launch finishes `count` edge cells or `count` corner cells.
template <typename S, bool ODD>
__global__ void surfaceKernel(DevLattice L, const int4* __restrict__ cells, int count, int pending,
                              typename StoreT<S>::R invRho0, double bbRho, typename StoreT<S>::R omega) {
    using R = typename StoreT<S>::R;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int4 c = cells[t];
    const long long idx = ((long long)c.x * L.ny + c.y) * L.nz + c.z;
    R rho, g[3][3], vel[3], f[19];
    surfaceGradientsAA<S, ODD>(L, c, pending, invRho0, bbRho, rho, g);
#pragma unroll
    for (int d = 0; d < 3; ++d) vel[d] = (R)L.bc[d * L.n + idx];
    surfaceFromGradients<R>(rho, g, vel, omega, f);
    Neighbourhood nb = neighbourhood(L, c.x, c.y, c.z);
    S* Pp = static_cast<S*>(L.pop);
#pragma unroll
    for (int i = 0; i < 19; ++i) StoreT<S>::st(Pp + slotOf<ODD>(L, nb, idx, i), f[i]);
}

// BoxRhoBarJfunctional3D (dataAnalysisFunctional3D.hh:528-549): each cell's
// Dynamics::computeRhoBarJ into the external-field planes (rho-bar, jx, jy,
// jz).  pending = 0 reads boundary faces as streamed (the functional running
// at a later processor level than the face completion); pending = 1 reads the
// completed state.
template <typename S, bool ODD>
__global__ void rhoBarJKernel(DevLattice L, int pending, double bbRho, typename StoreT<S>::F* out) {
    using R = typename StoreT<S>::R;
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    if (z >= L.nz) return;
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    const int k = L.flags[idx];
    if (k == K_NONE) return;
    R rb = R(0), j[3] = {R(0), R(0), R(0)};
    if (k == K_BB || k == K_MEBB) {  // core/dynamics.hh:880-885, bounceBackModels.hh:226-231
        rb = (R)bbRho - (R)1;
    } else if (k == K_NODYN) {       // core/dynamics.hh:1061-1066
        rb = (R)1 - (R)1;
    } else {
        Neighbourhood nb = neighbourhood(L, x, y, z);
        const S* Pp = static_cast<const S*>(L.pop);
        R f[19];
#pragma unroll
        for (int i = 0; i < 19; ++i) f[i] = StoreT<S>::ld(Pp + slotOf<ODD>(L, nb, idx, i));
        if (pending && isFace(k)) completeIfFace<R>(L, idx, k, f);
        if (k == K_BGK || k == K_GUO || k == K_INCBGK) {  // core/dynamics.hh:357-361
            rhoBarJ<R>(f, rb, j);
        } else if (isSurface(k)) {   // boundaryDynamics.hh:348-360
            const R rho = rhoBarSeq<R>(f) + (R)1;
            rb = rho - (R)1;
#pragma unroll
            for (int d = 0; d < 3; ++d) j[d] = rho * ((R)L.bc[d * L.n + idx] - (R)0.5 * (R)0);
        } else {                     // faces: boundaryDynamics.hh:682-702, 815-822
            const int fam = faceFamily(k), dir = faceDir(k);
            if (fam == 0 || fam == 2) {
                rb = velFaceRhoBarAny<R>(f, k, (R)L.bc[dir * L.n + idx]);
                const R rho = rb + (R)1;
#pragma unroll
                for (int d = 0; d < 3; ++d) j[d] = rho * ((R)L.bc[d * L.n + idx] - (R)0.5 * (R)0);
            } else {
                rb = (R)L.bc[idx] - (R)1;
                pressFaceJAny<R>(f, k, rb, j);
            }
        }
    }
    out[idx] = rb;
    out[L.n + idx] = j[0];
    out[2 * L.n + idx] = j[1];
    out[3 * L.n + idx] = j[2];
}

// computeAverageEnergy / computeAverageDensity (dataAnalysisWrapper3D.hh:1226-1262).
// Accumulation is in FP64.
template <typename S, bool ODD>
__global__ void reduceKernel(DevLattice L, Box b, int pending, typename StoreT<S>::R invRho0, double bbRho,
                             ReduceAcc* acc) {
    using R = typename StoreT<S>::R;
    const int bnz = b.z1 - b.z0 + 1;
    const int dz = blockIdx.x * blockDim.x + threadIdx.x;
    double e = 0., r = 0.;
    unsigned long long live = 0;
    if (dz < bnz) {
        R u[3], rb;
        double rho;
        if (cellMacroscopic<S, ODD>(L, b.x0 + blockIdx.z, b.y0 + blockIdx.y, b.z0 + dz, pending, invRho0, bbRho, u,
                                    rb, rho)) {
            e = (double)(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
            r = (double)rb;
            live = 1;
        }
    }
    // block sum, then one set of atomics per block on slot block % kStatsSlots
    __shared__ double shE[32], shR[32];
    __shared__ unsigned long long shL[32];
    e = warpSum(e);
    r = warpSum(r);
    live = warpSumU(live);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
        shE[w] = e;
        shR[w] = r;
        shL[w] = live;
    }
    __syncthreads();
    if (w == 0) {
        e = warpSum(lane < nw ? shE[lane] : 0.);
        r = warpSum(lane < nw ? shR[lane] : 0.);
        live = warpSumU(lane < nw ? shL[lane] : 0ull);
        if (lane == 0) {
            const unsigned b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
            ReduceAcc* a = acc + (b & (kStatsSlots - 1));
            atomicAdd(&a->sumEnergy, e);
            atomicAdd(&a->sumRhoBar, r);
            atomicAdd(&a->cells, live);
        }
    }
}

// computeVelocity (what = 0, 3 values per cell) / computeDensity (what = 1)
// (dataAnalysisWrapper3D.h:80-132) into a packed box buffer, FP64.
template <typename S, bool ODD>
__global__ void fieldKernel(DevLattice L, Box b, int pending, typename StoreT<S>::R invRho0, double bbRho, int what,
                            double* out) {
    using R = typename StoreT<S>::R;
    const int bnz = b.z1 - b.z0 + 1, bny = b.y1 - b.y0 + 1;
    const int dz = blockIdx.x * blockDim.x + threadIdx.x;
    if (dz >= bnz) return;
    const long long o = ((long long)blockIdx.z * bny + blockIdx.y) * bnz + dz;
    R u[3] = {R(0), R(0), R(0)}, rb = R(0);
    double rho = 0.;
    cellMacroscopic<S, ODD>(L, b.x0 + blockIdx.z, b.y0 + blockIdx.y, b.z0 + dz, pending, invRho0, bbRho, u, rb, rho);
    if (what == 0) {
        out[3 * o] = (double)u[0];
        out[3 * o + 1] = (double)u[1];
        out[3 * o + 2] = (double)u[2];
    } else {
        out[o] = rho;
    }
}

}  // namespace plbgpu
