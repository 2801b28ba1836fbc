// Interior-row step kernel of the 2-byte storage forms (BF16, BF16 with
// stochastic rounding, FP16): CPT = 2, 4 or 8 consecutive cells of a row per
// thread, every population read and written as one aligned 32-, 64- or
// 128-bit word, the populations of all CPT cells held packed (one register
// per two cells and population) while the cells collide one after another.
//
// Rows with 1 <= x <= nx-2 and 1 <= y <= ny-2 of a dense domain whose rows
// hold a multiple of CPT cells (planes start on 256-byte boundaries, so every
// CPT-cell segment of a plane row is one aligned vector).  Thread g owns
// segment g % (nz/CPT) of interior row g / (nz/CPT): cells z0..z0+CPT-1,
// z0 = CPT * segment.
//
// Even AA step: the 19 vectors of the thread's own cells are loaded, each
// cell collides, and population i goes back into slot opp(i) of the same
// cells -- 19 vector loads and 19 vector stores per eight cells.
//
// Odd AA step: slot opp(i) of x - c_i is read and population i written to slot
// i of x + c_i.  Moves along x and y are a uniform row offset (interior rows);
// the nine populations with c_z = 0 stay aligned.  For the ten that move along
// z the thread's window is its aligned vector shifted by one cell: the missing
// element is the neighbouring lane's edge element, passed by one warp shuffle
// and merged with four byte permutes.  Where the neighbour is not in the same
// row and warp the element is read with a 16-bit load: at a warp boundary
// inside a row, the plain neighbour; at the row ends, the periodic wrap or --
// on a non-periodic z axis -- the reference's domain-edge rule (a population
// that would leave the domain stays in its cell, reversed: slot i of the own
// cell).  Stores mirror this: a lane whose vector needs an element from a lane
// it cannot shuffle with writes its other CPT - 1 elements with 16-, 32- and
// 64-bit stores, and the element's owner writes it with a 16-bit store.
//
// Every slot is still read and written by one thread only: an element a
// thread hands to its neighbour through a shuffle is one the thread itself
// read, and an element it receives is one it writes.  This is the same
// ownership as the one-cell kernels, so the results are bit-identical to them.
#pragma once

#include "kernels.cuh"

namespace plbgpu {

// Unpack one 16-bit value (low or high half of a 32-bit word) to FP32 and pack
// an FP32 value into one half of a word, per storage type.
template <typename S> struct Half16;
template <> struct Half16<__nv_bfloat16> {
    static __device__ __forceinline__ float get(unsigned w, bool hi) {
        return __uint_as_float(hi ? (w & 0xffff0000u) : (w << 16));
    }
    static __device__ __forceinline__ unsigned put(unsigned w, bool hi, float v, const void*, unsigned) {
        const unsigned b = __bfloat16_as_ushort(__float2bfloat16_rn(v));
        return hi ? __byte_perm(w, b, 0x5410) : __byte_perm(w, b, 0x3254);
    }
};
template <> struct Half16<__half> {
    static __device__ __forceinline__ float get(unsigned w, bool hi) {
        return __half2float(__ushort_as_half((unsigned short)(hi ? (w >> 16) : (w & 0xffffu))));
    }
    static __device__ __forceinline__ unsigned put(unsigned w, bool hi, float v, const void*, unsigned) {
        const unsigned b = __half_as_ushort(__float2half_rn(v));
        return hi ? __byte_perm(w, b, 0x5410) : __byte_perm(w, b, 0x3254);
    }
};
template <> struct Half16<bf16sr> {
    static __device__ __forceinline__ float get(unsigned w, bool hi) {
        return __uint_as_float(hi ? (w & 0xffff0000u) : (w << 16));
    }
    // random bits from the cell's own slot address and the step's salt
    static __device__ __forceinline__ unsigned put(unsigned w, bool hi, float v, const void* cellSlot, unsigned salt) {
        const unsigned b = bf16Stochastic(v, srBits(cellSlot, salt));
        return hi ? __byte_perm(w, b, 0x5410) : __byte_perm(w, b, 0x3254);
    }
};

// NW 32-bit words of 16-bit values (NW = 1, 2 or 4: four, eight or sixteen
// bytes), element e in word e / 2, low half first.
template <int NW>
struct Words {
    unsigned w[NW];
};

template <int NW>
__device__ __forceinline__ Words<NW> ldWords(const void* p) {
    Words<NW> v;
    if constexpr (NW == 4)
        asm volatile("ld.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                     : "=r"(v.w[0]), "=r"(v.w[1]), "=r"(v.w[2]), "=r"(v.w[3])
                     : "l"(p));
    else if constexpr (NW == 2)
        asm volatile("ld.global.v2.u32 {%0, %1}, [%2];" : "=r"(v.w[0]), "=r"(v.w[1]) : "l"(p));
    else   // a warp reads 128 bytes of a plane: the L2 prefetches the 256-byte segment
        v.w[0] = ldPair256(p);
    return v;
}
template <int NW>
__device__ __forceinline__ void stWords(void* p, const Words<NW>& v) {
    if constexpr (NW == 4)
        asm volatile("st.global.v4.u32 [%0], {%1, %2, %3, %4};" ::"l"(p), "r"(v.w[0]), "r"(v.w[1]), "r"(v.w[2]),
                     "r"(v.w[3])
                     : "memory");
    else if constexpr (NW == 2)
        asm volatile("st.global.v2.u32 [%0], {%1, %2};" ::"l"(p), "r"(v.w[0]), "r"(v.w[1]) : "memory");
    else
        asm volatile("st.global.u32 [%0], %1;" ::"l"(p), "r"(v.w[0]) : "memory");
}
__device__ __forceinline__ unsigned ld16(const void* p) {
    unsigned short u;
    asm volatile("ld.global.u16 %0, [%1];" : "=h"(u) : "l"(p));
    return u;
}
__device__ __forceinline__ void st16(void* p, unsigned v) {
    asm volatile("st.global.u16 [%0], %1;" ::"l"(p), "h"((unsigned short)v) : "memory");
}
__device__ __forceinline__ void st32(void* p, unsigned v) {
    asm volatile("st.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st64(void* p, unsigned a, unsigned b) {
    asm volatile("st.global.v2.u32 [%0], {%1, %2};" ::"l"(p), "r"(a), "r"(b) : "memory");
}

// (p, e0, ..., e_{n-2}): p in the high half of `prev`.
template <int NW>
__device__ __forceinline__ Words<NW> shiftUp(const Words<NW>& v, unsigned prev) {
    Words<NW> r;
    r.w[0] = __byte_perm(prev, v.w[0], 0x5432);
#pragma unroll
    for (int k = 1; k < NW; ++k) r.w[k] = __byte_perm(v.w[k - 1], v.w[k], 0x5432);
    return r;
}
// (e1, ..., e_{n-1}, n): n in the low half of `next`.
template <int NW>
__device__ __forceinline__ Words<NW> shiftDown(const Words<NW>& v, unsigned next) {
    Words<NW> r;
#pragma unroll
    for (int k = 0; k + 1 < NW; ++k) r.w[k] = __byte_perm(v.w[k], v.w[k + 1], 0x5432);
    r.w[NW - 1] = __byte_perm(v.w[NW - 1], next, 0x5432);
    return r;
}

// Uniform row offsets c_x * ny * nz + c_y * nz of the 19 populations.
struct RowDeltas {
    int d[19];
};

// Cells per thread and residency of the vector kernel: CPT = 8 moves 16-byte
// vectors (19 of them held as 76 registers of packed values), CPT = 4 moves
// 8-byte vectors with half the registers and more resident warps, CPT = 2
// 4-byte words (19 registers of packed values, 64 registers a thread).
template <int CPT>
struct VecShape {
    static constexpr int blocks = CPT == 8 ? 3 : CPT == 4 ? 5 : 8;
};

template <typename S, bool ODD, bool STATS, bool EXT, int CPT>
__global__ void __launch_bounds__(128, VecShape<CPT>::blocks)
    vecRowStepKernel(DevLattice L, Planes<S> Pl, RowDeltas D, StepParams<typename StoreT<S>::R> P, StatsAcc* acc,
                     long long segments) {
    using R = typename StoreT<S>::R;
    constexpr int NW = CPT / 2;
    const int RS = L.nz / CPT;                      // segments per row
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = g < segments;
    // Threads past the last segment mirror it (the warp's shuffles need every
    // lane); they store nothing and gather no statistics.
    const long long gg = live ? g : segments - 1;
    int x, y, z0;
    bool live2 = live, upOk, downOk;
    const int lane = threadIdx.x & 31;
    if (L.denseTiles) {   // sparse domain: segments of the dense tiles
        constexpr int TS = kTileCells / CPT;
        const int r = (int)(gg / TS), s = (int)(gg - (long long)r * TS);
        const int4 t = L.denseTiles[r];
        x = t.x;
        y = t.y;
        z0 = t.z + s * CPT;
        if (z0 >= t.w) {  // past a short tile's end: mirror its first segment
            z0 = t.z;
            live2 = false;
        }
        upOk = s > 0 && lane > 0;
        downOk = s + 1 < TS && z0 + CPT < t.w && lane < 31;
    } else {
        const int row = (int)(gg / RS), seg = (int)(gg - (long long)row * RS);
        x = 1 + L.xRow0 + row / (L.ny - 2);
        y = 1 + row % (L.ny - 2);
        z0 = seg * CPT;
        upOk = seg > 0 && lane > 0;                 // lane - 1 holds the CPT cells below z0 in this row
        downOk = seg < RS - 1 && lane < 31;         // lane + 1 holds the CPT cells from z0 + CPT on
    }
    const int nz = L.nz;
    const bool first = z0 == 0, last = z0 + CPT == nz;
    const bool perZ = L.per[2] != 0;
    const int rowIdx = (x * L.ny + y) * nz;
    const int idx0 = rowIdx + z0;

    Words<NW> v[19];
    // ---- load
#pragma unroll
    for (int i = 0; i < 19; ++i) {
        if (!ODD) {
            v[i] = ldWords<NW>(Pl.p[i] + idx0);
        } else {
            const S* src = Pl.p[opp(i)];
            const int srow = rowIdx - D.d[i];       // source row x - c_i (x and y part)
            const int cz = cdir(i, 2);
            const Words<NW> a = ldWords<NW>(src + (srow + z0));
            if (cz == 0) {
                v[i] = a;
            } else if (cz > 0) {                    // window z0-1 .. z0+CPT-2
                unsigned prev = __shfl_up_sync(0xffffffffu, a.w[NW - 1], 1);
                if (!upOk) {
                    const S* p = !first ? src + (srow + z0 - 1) : (perZ ? src + (srow + nz - 1) : Pl.p[i] + rowIdx);
                    prev = ld16(p) << 16;
                }
                v[i] = shiftUp<NW>(a, prev);
            } else {                                // window z0+1 .. z0+CPT
                unsigned next = __shfl_down_sync(0xffffffffu, a.w[0], 1);
                if (!downOk) {
                    const S* p = !last ? src + (srow + z0 + CPT) : (perZ ? src + srow : Pl.p[i] + (rowIdx + nz - 1));
                    next = ld16(p);
                }
                v[i] = shiftDown<NW>(a, next);
            }
        }
    }
    unsigned kk[2];   // the cells' kinds, four per word
    if constexpr (NW == 4) {
        const uint2 t = *reinterpret_cast<const uint2*>(L.flags + idx0);
        kk[0] = t.x;
        kk[1] = t.y;
    } else if constexpr (NW == 2) {
        kk[0] = *reinterpret_cast<const unsigned*>(L.flags + idx0);
        kk[1] = 0u;
    } else {
        kk[0] = *reinterpret_cast<const unsigned short*>(L.flags + idx0);
        kk[1] = 0u;
    }

    // ---- collide, one cell at a time; results go back into the same halves
    double sR = 0., sU = 0.;
    unsigned long long cnt = 0, mx = 0;
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
        const int w = c >> 1;
        const bool hi = c & 1;
        const int k = (int)((kk[c >> 2] >> (8 * (c & 3))) & 0xffu);
        R f[19];
#pragma unroll
        for (int i = 0; i < 19; ++i) f[i] = Half16<S>::get(v[i].w[w], hi);
        const int idx = idx0 + c;
        R rhoBar = R(0), uSqr = R(0);
        if (P.pending && !L.rowFacesDone && isFace(k)) completeIfFace<R>(L, idx, k, f);
        const bool gathers = collideCell<S, EXT>(L, P, idx, k, f, rhoBar, uSqr, acc, STATS && live2);
#pragma unroll
        for (int i = 0; i < 19; ++i) v[i].w[w] = Half16<S>::put(v[i].w[w], hi, f[i], Pl.p[i] + idx, P.seed);
        if (STATS && live2 && gathers) {
            sR += (double)rhoBar;
            sU += (double)uSqr;
            cnt += 1;
            const unsigned long long b = (unsigned long long)__double_as_longlong((double)uSqr);
            mx = b > mx ? b : mx;
        }
    }

    // ---- store
#pragma unroll
    for (int i = 0; i < 19; ++i) {
        if (!ODD) {
            if (live2) stWords<NW>(Pl.p[opp(i)] + idx0, v[i]);
        } else {
            S* dst = Pl.p[i];
            const int drow = rowIdx + D.d[i];       // destination row x + c_i (x and y part)
            const int d0 = drow + z0;
            const int cz = cdir(i, 2);
            const Words<NW>& a = v[i];
            if (cz == 0) {
                if (live2) stWords<NW>(dst + d0, a);
            } else if (cz > 0) {                    // cells z0.. -> positions z0+1 .. z0+CPT
                const unsigned prev = __shfl_up_sync(0xffffffffu, a.w[NW - 1], 1);
                if (live2) {
                    if (upOk) {
                        stWords<NW>(dst + d0, shiftUp<NW>(a, prev));
                    } else {                        // position z0 is written by its owner
                        st16(dst + (d0 + 1), a.w[0]);
                        if constexpr (NW >= 2) st32(dst + (d0 + 2), __byte_perm(a.w[0], a.w[1], 0x5432));
                        if constexpr (NW == 4)
                            st64(dst + (d0 + 4), __byte_perm(a.w[1], a.w[2], 0x5432),
                                 __byte_perm(a.w[2], a.w[3], 0x5432));
                    }
                    if (!downOk) {                  // the last cell's value: no lane of this warp takes it
                        S* p = !last ? dst + (d0 + CPT) : (perZ ? dst + drow : Pl.p[opp(i)] + (rowIdx + nz - 1));
                        st16(p, a.w[NW - 1] >> 16);
                    }
                }
            } else {                                // cells z0.. -> positions z0-1 .. z0+CPT-2
                const unsigned next = __shfl_down_sync(0xffffffffu, a.w[0], 1);
                if (live2) {
                    if (downOk) {
                        stWords<NW>(dst + d0, shiftDown<NW>(a, next));
                    } else {                        // position z0+CPT-1 is written by its owner
                        if constexpr (NW == 4) {
                            st64(dst + d0, __byte_perm(a.w[0], a.w[1], 0x5432), __byte_perm(a.w[1], a.w[2], 0x5432));
                            st32(dst + (d0 + 4), __byte_perm(a.w[2], a.w[3], 0x5432));
                        } else if constexpr (NW == 2) {
                            st32(dst + d0, __byte_perm(a.w[0], a.w[1], 0x5432));
                        }
                        st16(dst + (d0 + CPT - 2), a.w[NW - 1] >> 16);
                    }
                    if (!upOk) {                    // the first cell's value: no lane of this warp takes it
                        S* p = !first ? dst + (d0 - 1) : (perZ ? dst + (drow + nz - 1) : Pl.p[opp(i)] + rowIdx);
                        st16(p, a.w[0]);
                    }
                }
            }
        }
    }
    if (STATS) flushStats(sR, sU, cnt, mx, acc, L.status);
}

}  // namespace plbgpu
