// D3Q19 per-cell arithmetic for the fused collide-and-stream kernels.
//
// Every expression keeps the operand order of the reference's templates so
// that, in FP64 and compiled without FMA contraction, the device produces the
// same bits as the reference CPU path.  The same code instantiated with
// R = float is the FP32-compute form.  Citations are to the reference's src/.
#pragma once

#include <utility>

#include <cstdint>
#include <cuda_runtime.h>

namespace plbgpu {

// latticeBoltzmann/nearestNeighborLattices3D.hh:168-180
__device__ constexpr int CX[19] = {0, -1, 0, 0, -1, -1, -1, -1, 0, 0, 1, 0, 0, 1, 1, 1, 1, 0, 0};
__device__ constexpr int CY[19] = {0, 0, -1, 0, -1, 1, 0, 0, -1, -1, 0, 1, 0, 1, -1, 0, 0, 1, 1};
__device__ constexpr int CZ[19] = {0, 0, 0, -1, 0, 0, -1, 1, -1, 1, 0, 0, 1, 0, 0, 1, -1, 1, -1};

__host__ __device__ constexpr int opp(int i) { return i == 0 ? 0 : (i <= 9 ? i + 9 : i - 9); }
__host__ __device__ constexpr int cdir(int i, int d) {
    return d == 0 ? (i == 0 ? 0 : (i == 1 || i == 4 || i == 5 || i == 6 || i == 7) ? -1
                                  : (i == 10 || i == 13 || i == 14 || i == 15 || i == 16) ? 1 : 0)
         : d == 1 ? (i == 2 || i == 4 || i == 8 || i == 9 || i == 14) ? -1
                    : (i == 5 || i == 11 || i == 13 || i == 17 || i == 18) ? 1 : 0
                  : (i == 3 || i == 6 || i == 8 || i == 16 || i == 18) ? -1
                    : (i == 7 || i == 9 || i == 12 || i == 15 || i == 17) ? 1 : 0;
}
__host__ __device__ constexpr int cnorm2(int i) {
    return cdir(i, 0) * cdir(i, 0) + cdir(i, 1) * cdir(i, 1) + cdir(i, 2) * cdir(i, 2);
}

// Cell kinds (one byte per cell).
enum Kind : uint8_t {
    K_BGK = 0, K_GUO = 1, K_INCBGK = 2, K_BB = 3, K_MEBB = 4, K_NODYN = 5,
    K_REGVEL = 6, K_REGPRESS = 12, K_ZHVEL = 18, K_ZHPRESS = 24,
    K_EDGE = 30,    // 30..41: external velocity edge, 30 + 4*plane + 2*(normal1>0) + (normal2>0)
    K_CORNER = 42,  // 42..49: external velocity corner, 42 + 4*(xNormal>0) + 2*(yNormal>0) + (zNormal>0)
    K_NKINDS = 50,
    K_NONE = 255  // not part of the lattice (sparse storage)
};
__host__ __device__ inline bool isFace(int k) { return k >= K_REGVEL && k < K_EDGE; }
// Edge and corner cells: StoreVelocityDynamics around the BGK base, finished
// after each step by the finite-difference processors.
__host__ __device__ inline bool isSurface(int k) { return k >= K_EDGE && k < K_NKINDS; }
// Kinds that collide with the plain BGK rule.
__host__ __device__ inline bool bgkBase(int k) { return k == K_BGK || (k >= K_REGVEL && k < K_NKINDS); }
__host__ __device__ inline int faceFamily(int k) { return (k - K_REGVEL) / 6; }
__host__ __device__ inline int faceDir(int k) { return ((k - K_REGVEL) % 6) / 2; }
__host__ __device__ inline int faceOri(int k) { return (((k - K_REGVEL) % 6) % 2) ? 1 : -1; }
// Kinds whose collision gathers the lattice statistics (latticeStatistics.h:38-43).
__host__ __device__ inline bool takesStats(int k) { return k == K_GUO || k == K_INCBGK || bgkBase(k); }

// Lattice weights, computed as (T)1/(T)3 etc. (nearestNeighborLattices3D.hh:183-205).
template <typename R>
__device__ __forceinline__ R tw(int i) {
    return i == 0 ? (R)1 / (R)3 : (cnorm2(i) == 1 ? (R)1 / (R)18 : (R)1 / (R)36);
}

// 1 / (rhoBar + 1) (roundOffPolicy.h:85-87).  The round-to-nearest reciprocal
// intrinsics return the correctly rounded quotient, i.e. the same bits as the
// IEEE division 1/x.
__device__ __forceinline__ double invRhoOf(double rhoBar) { return __drcp_rn(rhoBar + 1.0); }
__device__ __forceinline__ float invRhoOf(float rhoBar) { return __frcp_rn(rhoBar + 1.0f); }

// momentTemplates3D.h:351-365, 411-425
template <typename R>
__device__ __forceinline__ void rhoBarJ(const R* f, R& rhoBar, R* j) {
    R sxm = f[1] + f[4] + f[5] + f[6] + f[7];
    R sxp = f[10] + f[13] + f[14] + f[15] + f[16];
    R sym = f[2] + f[4] + f[8] + f[9] + f[14];
    R syp = f[5] + f[11] + f[13] + f[17] + f[18];
    R szm = f[3] + f[6] + f[8] + f[16] + f[18];
    R szp = f[7] + f[9] + f[12] + f[15] + f[17];
    R sx0 = f[0] + f[2] + f[3] + f[8] + f[9] + f[11] + f[12] + f[17] + f[18];
    rhoBar = sxm + sx0 + sxp;
    j[0] = sxp - sxm;
    j[1] = syp - sym;
    j[2] = szp - szm;
}

// momentTemplates3D.h:372-379 (sequential 19-term sum)
template <typename R>
__device__ __forceinline__ R rhoBarSeq(const R* f) {
    R r = f[0];
#pragma unroll
    for (int i = 1; i < 19; ++i) r = r + f[i];
    return r;
}

// dynamicsTemplates3D.h:1994-1997; c.j sums only the non-zero terms in the
// reference's order (the dropped terms are signed zeros).
template <typename R>
__device__ __forceinline__ R cDotJ(int i, const R* j) {
    R s = R(0);
    bool first = true;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int c = cdir(i, d);
        if (c == 0) continue;
        R t = (c > 0) ? j[d] : -j[d];
        s = first ? t : s + t;
        first = false;
    }
    return s;
}

template <typename R>
__device__ __forceinline__ R bgkEq(int i, R rhoBar, R invRho, const R* j, R jSqr) {
    R cj = cDotJ<R>(i, j);
    return tw<R>(i) * (rhoBar + (R)3. * cj + invRho * ((R)4.5 * cj * cj - (R)1.5 * jSqr));
}

// Precomputed per-launch constants of bgk_ma2_collision_base.
template <typename R>
struct BgkConst {
    R omega, one_m_omega, t0_omega, t1_omega, t4_omega;
};

// dynamicsTemplates3D.h:2289-2366
template <typename R>
__device__ __forceinline__ R bgkCollide(R* f, R rhoBar, const R* j, const BgkConst<R>& k, R invRho) {
    const R om1 = k.one_m_omega, t0 = k.t0_omega, t1 = k.t1_omega, t4 = k.t4_omega;
    R jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    R kx = (R)3 * j[0];
    R ky = (R)3 * j[1];
    R kz = (R)3 * j[2];
    R half = invRho / (R)2;
    R kxSqr_ = half * kx * kx;
    R kySqr_ = half * ky * ky;
    R kzSqr_ = half * kz * kz;
    R kxky_ = invRho * kx * ky;
    R kxkz_ = invRho * kx * kz;
    R kykz_ = invRho * ky * kz;
    R C1 = rhoBar + invRho * (R)3 * jSqr;
    R C2, C3;
    C3 = -kxSqr_ - kySqr_ - kzSqr_;
    f[0] *= om1; f[0] += t0 * (C1 + C3);
    C2 = -kx; C3 = -kySqr_ - kzSqr_;
    f[1] *= om1; f[1] += t1 * (C1 + C2 + C3);
    f[10] *= om1; f[10] += t1 * (C1 - C2 + C3);
    C2 = -ky; C3 = -kxSqr_ - kzSqr_;
    f[2] *= om1; f[2] += t1 * (C1 + C2 + C3);
    f[11] *= om1; f[11] += t1 * (C1 - C2 + C3);
    C2 = -kz; C3 = -kxSqr_ - kySqr_;
    f[3] *= om1; f[3] += t1 * (C1 + C2 + C3);
    f[12] *= om1; f[12] += t1 * (C1 - C2 + C3);
    C2 = -kx - ky; C3 = kxky_ - kzSqr_;
    f[4] *= om1; f[4] += t4 * (C1 + C2 + C3);
    f[13] *= om1; f[13] += t4 * (C1 - C2 + C3);
    C2 = -kx + ky; C3 = -kxky_ - kzSqr_;
    f[5] *= om1; f[5] += t4 * (C1 + C2 + C3);
    f[14] *= om1; f[14] += t4 * (C1 - C2 + C3);
    C2 = -kx - kz; C3 = kxkz_ - kySqr_;
    f[6] *= om1; f[6] += t4 * (C1 + C2 + C3);
    f[15] *= om1; f[15] += t4 * (C1 - C2 + C3);
    C2 = -kx + kz; C3 = -kxkz_ - kySqr_;
    f[7] *= om1; f[7] += t4 * (C1 + C2 + C3);
    f[16] *= om1; f[16] += t4 * (C1 - C2 + C3);
    C2 = -ky - kz; C3 = kykz_ - kxSqr_;
    f[8] *= om1; f[8] += t4 * (C1 + C2 + C3);
    f[17] *= om1; f[17] += t4 * (C1 - C2 + C3);
    C2 = -ky + kz; C3 = -kykz_ - kxSqr_;
    f[9] *= om1; f[9] += t4 * (C1 + C2 + C3);
    f[18] *= om1; f[18] += t4 * (C1 - C2 + C3);
    return invRho * invRho * jSqr;
}

// externalForceTemplates3D.h:73-150 (ForcedD3Q19, amplitude 1)
template <typename R>
__device__ __forceinline__ void addGuoForce(R* f, const R* F, const R* u, R omega) {
    const R mu = (R)1 * ((R)1 - omega / (R)2);
    const R o6 = (R)1 / (R)6;
    const R o12 = (R)1 / (R)12;
    const R one = (R)1;
    f[0] += -mu * (F[0] * u[0] + F[1] * u[1] + F[2] * u[2]);
    f[1] += o6 * mu * (F[0] * (-one + (R)2 * u[0]) - F[1] * u[1] - F[2] * u[2]);
    f[2] += -o6 * mu * (F[0] * u[0] + F[1] * (one - (R)2 * u[1]) + F[2] * u[2]);
    f[3] += -o6 * mu * (F[0] * u[0] + F[1] * u[1] + F[2] * (one - (R)2 * u[2]));
    f[4] += o12 * mu * (F[0] * (-one + (R)2 * u[0] + (R)3 * u[1]) + F[1] * (-one + (R)2 * u[1] + (R)3 * u[0]) - F[2] * u[2]);
    f[5] += o12 * mu * (F[0] * (-one + (R)2 * u[0] - (R)3 * u[1]) + F[1] * (one + (R)2 * u[1] - (R)3 * u[0]) - F[2] * u[2]);
    f[6] += o12 * mu * (F[0] * (-one + (R)2 * u[0] + (R)3 * u[2]) - F[1] * u[1] + F[2] * (-one + (R)2 * u[2] + (R)3 * u[0]));
    f[7] += o12 * mu * (F[0] * (-one + (R)2 * u[0] - (R)3 * u[2]) - F[1] * u[1] + F[2] * (one + (R)2 * u[2] - (R)3 * u[0]));
    f[8] += -o12 * mu * (F[0] * u[0] + F[1] * (one - (R)2 * u[1] - (R)3 * u[2]) + F[2] * (one - (R)2 * u[2] - (R)3 * u[1]));
    f[9] += -o12 * mu * (F[0] * u[0] + F[1] * (one - (R)2 * u[1] + (R)3 * u[2]) + F[2] * (-one - (R)2 * u[2] + (R)3 * u[1]));
    f[10] += o6 * mu * (F[0] * (one + (R)2 * u[0]) - F[1] * u[1] - F[2] * u[2]);
    f[11] += -o6 * mu * (F[0] * u[0] + F[1] * (-one - (R)2 * u[1]) + F[2] * u[2]);
    f[12] += -o6 * mu * (F[0] * u[0] + F[1] * u[1] + F[2] * (-one - (R)2 * u[2]));
    f[13] += o12 * mu * (F[0] * (one + (R)2 * u[0] + (R)3 * u[1]) + F[1] * (one + (R)2 * u[1] + (R)3 * u[0]) - F[2] * u[2]);
    f[14] += o12 * mu * (F[0] * (one + (R)2 * u[0] - (R)3 * u[1]) + F[1] * (-one + (R)2 * u[1] - (R)3 * u[0]) - F[2] * u[2]);
    f[15] += o12 * mu * (F[0] * (one + (R)2 * u[0] + (R)3 * u[2]) - F[1] * u[1] + F[2] * (one + (R)2 * u[2] + (R)3 * u[0]));
    f[16] += o12 * mu * (F[0] * (one + (R)2 * u[0] - (R)3 * u[2]) - F[1] * u[1] + F[2] * (-one + (R)2 * u[2] - (R)3 * u[0]));
    f[17] += -o12 * mu * (F[0] * u[0] + F[1] * (-one - (R)2 * u[1] - (R)3 * u[2]) + F[2] * (-one - (R)2 * u[2] - (R)3 * u[1]));
    f[18] += -o12 * mu * (F[0] * u[0] + F[1] * (-one - (R)2 * u[1] + (R)3 * u[2]) + F[2] * (one - (R)2 * u[2] + (R)3 * u[1]));
}

// ---------------------------------------------------------------- boundary faces
//
// The wrapped regularized / Zou-He face conditions complete a boundary cell's
// populations after streaming (wrappedLocalBoundaryProcessor3D.hh:43-65).  The
// kernels apply the completion when the cell is loaded for the next collision
// (and when the state is read back), which is the same sequence of operations.

// The direction and orientation of a face are template parameters, so every
// loop over the populations unrolls with compile-time index sets.

// i-th population (ascending) with c[DIR] == VAL (indexTemplates.h:81-97).
template <int DIR, int VAL>
__host__ __device__ constexpr int subIndex(int a) {
    int n = 0;
    for (int i = 0; i < 19; ++i)
        if (cdir(i, DIR) == VAL) {
            if (n == a) return i;
            ++n;
        }
    return -1;
}
template <int DIR, int VAL>
__host__ __device__ constexpr int subIndexCount() {
    int n = 0;
    for (int i = 0; i < 19; ++i) n += (cdir(i, DIR) == VAL) ? 1 : 0;
    return n;
}

// A population index known at compile time.
template <int I>
struct Idx {
    __host__ __device__ constexpr operator int() const { return I; }
};

// fn(i) for each population i with c[DIR] == VAL, ascending, i a compile-time
// constant (Idx): the index set is evaluated by the C++ front end, not by
// unrolling subIndex's search in the optimizer.
template <int DIR, int VAL, typename Fn, int... A>
__device__ __forceinline__ void forSubImpl(Fn& fn, std::integer_sequence<int, A...>) {
    (fn(Idx<subIndex<DIR, VAL>(A)>()), ...);
}
template <int DIR, int VAL, typename Fn>
__device__ __forceinline__ void forSub(Fn&& fn) {
    forSubImpl<DIR, VAL>(fn, std::make_integer_sequence<int, subIndexCount<DIR, VAL>()>());
}

// boundaryDynamics.hh:639-669 (VelocityDirichletBoundaryDynamics::computeRhoBar)
template <typename R, int DIR, int ORI>
__device__ __forceinline__ R velFaceRhoBar(const R* f, R velDir) {
    R rhoOnWall = R(0), rhoNormal = R(0);
    forSub<DIR, 0>([&](auto i) { rhoOnWall += f[i]; });
    forSub<DIR, ORI>([&](auto i) { rhoNormal += f[i]; });
    R velNormal = (R)ORI * (velDir - (R)0.5 * (R)0);
    return ((R)2 * rhoNormal + rhoOnWall - (R)1 * velNormal) / ((R)1 + velNormal);
}

// boundaryDynamics.hh:775-800 (DensityDirichletBoundaryDynamics::computeJ)
template <typename R, int DIR, int ORI>
__device__ __forceinline__ void pressFaceJ(const R* f, R rhoBar, R* j) {
    R rhoOnWall = R(0), rhoNormal = R(0);
    forSub<DIR, 0>([&](auto i) { rhoOnWall += f[i]; });
    forSub<DIR, ORI>([&](auto i) { rhoNormal += f[i]; });
    j[0] = j[1] = j[2] = R(0);
    j[DIR] = (R)ORI * ((R)2 * rhoNormal + rhoOnWall - rhoBar);
}

// offEquilibriumTemplates.h:91-115
template <typename R>
__device__ __forceinline__ R piToFneq(int i, const R* Pi) {
    R fNeq = R(0);
    int iPi = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        fNeq += Pi[iPi] * ((R)(cdir(i, a) * cdir(i, a)) - (R)1 / (R)3);
        ++iPi;
#pragma unroll
        for (int b = a + 1; b < 3; ++b) {
            fNeq += Pi[iPi] * (R)2 * (R)cdir(i, a) * (R)cdir(i, b);
            ++iPi;
        }
    }
    fNeq *= tw<R>(i) * (R)3 * (R)3 / (R)2;
    return fNeq;
}

// regularizedBoundaryDynamics.hh:96-110 with boundaryTemplates.h:42-84 and
// isoThermalDynamics.hh:55-69
// IsoThermalBulkDynamics::regularize with the BGK equilibrium
// (isoThermalDynamics.hh:55-69): f = f_eq(rhoBar, j) + fromPiToFneq(Pi).
template <typename R>
__device__ __forceinline__ void regularizeFromPi(R* f, R rhoBar, const R* j, R jSqr, const R* Pi) {
    R invRho = invRhoOf(rhoBar);
    f[0] = bgkEq<R>(0, rhoBar, invRho, j, jSqr) + piToFneq<R>(0, Pi);
#pragma unroll
    for (int i = 1; i <= 9; ++i) {
        f[i] = bgkEq<R>(i, rhoBar, invRho, j, jSqr);
        f[i + 9] = bgkEq<R>(i + 9, rhoBar, invRho, j, jSqr);
        R fn = piToFneq<R>(i, Pi);
        f[i] += fn;
        f[i + 9] += fn;
    }
}

template <typename R, int DIR, int ORI>
__device__ __forceinline__ void regularizedComplete(R* f, R rhoBar, const R* j) {
    R jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    R invRho = invRhoOf(rhoBar);
    R fNeq[19];
#pragma unroll
    for (int i = 0; i < 19; ++i) {
        const int c = cdir(i, DIR);
        fNeq[i] = (c == 0 || (c == ORI && i != 0)) ? f[i] - bgkEq<R>(i, rhoBar, invRho, j, jSqr) : R(0);
    }
    R Pi[6];
    int iPi = 0;
#pragma unroll
    for (int al = 0; al < 3; ++al)
#pragma unroll
        for (int be = al; be < 3; ++be) {
            R s = R(0);
            forSub<DIR, 0>([&](auto i) { s += (R)(cdir(i, al) * cdir(i, be)) * fNeq[i]; });
            forSub<DIR, ORI>([&](auto i) { s += (R)2 * (R)cdir(i, al) * (R)cdir(i, be) * fNeq[i]; });
            Pi[iPi++] = s;
        }
    f[0] = bgkEq<R>(0, rhoBar, invRho, j, jSqr) + piToFneq<R>(0, Pi);
#pragma unroll
    for (int i = 1; i <= 9; ++i) {
        f[i] = bgkEq<R>(i, rhoBar, invRho, j, jSqr);
        f[i + 9] = bgkEq<R>(i + 9, rhoBar, invRho, j, jSqr);
        R fn = piToFneq<R>(i, Pi);
        f[i] += fn;
        f[i + 9] += fn;
    }
}

// Missing populations of a Zou/He face: opposites of the c[DIR]==ORI set
// (indexTemplates.h:110-133), and the same list without the first population
// that has a single non-zero component (zouHeDynamics.hh:58-71).
template <int DIR, int ORI>
__host__ __device__ constexpr int zhMissing(int a) { return opp(subIndex<DIR, ORI>(a)); }
template <int DIR, int ORI>
__host__ __device__ constexpr int zhDiag(int a) {
    int n = 0;
    bool erased = false;
    for (int b = 0; b < subIndexCount<DIR, ORI>(); ++b) {
        int p = zhMissing<DIR, ORI>(b);
        if (!erased && cnorm2(p) == 1) { erased = true; continue; }
        if (n == a) return p;
        ++n;
    }
    return -1;
}

// fn(p) over zhMissing (DIAG false) or zhDiag (DIAG true), p a compile-time constant.
template <int DIR, int ORI, bool DIAG, typename Fn, int... A>
__device__ __forceinline__ void forEachZhImpl(Fn& fn, std::integer_sequence<int, A...>) {
    (fn(Idx<DIAG ? zhDiag<DIR, ORI>(A) : zhMissing<DIR, ORI>(A)>()), ...);
}
template <int DIR, int ORI, bool DIAG, typename Fn>
__device__ __forceinline__ void forEachZh(Fn&& fn) {
    constexpr int n = subIndexCount<DIR, ORI>() - (DIAG ? 1 : 0);
    forEachZhImpl<DIR, ORI, DIAG>(fn, std::make_integer_sequence<int, n>());
}

// zouHeDynamics.hh:44-113 (ZouHeClosure)
template <typename R, int DIR, int ORI>
__device__ __forceinline__ void zouHeComplete(R* f, R rhoBar, const R* j) {
    constexpr int nd = subIndexCount<DIR, ORI>() - 1;
    R jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    R invRho = invRhoOf(rhoBar);
    forEachZh<DIR, ORI, false>([&](auto p) {
        const int o = opp(p);
        f[p] = f[o] - bgkEq<R>(o, rhoBar, invRho, j, jSqr) + bgkEq<R>(p, rhoBar, invRho, j, jSqr);
    });
    R rb, jj[3];
    rhoBarJ<R>(f, rb, jj);
    R invR = invRhoOf(rb);
    R falseRho = rb + (R)1;
    R diff[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) diff[d] = (j[d] - falseRho * (jj[d] * invR)) / (R)nd;
    forEachZh<DIR, ORI, true>([&](auto p) {
#pragma unroll
        for (int s = 1; s < 3; ++s) {
            const int d = (DIR + s) % 3;
            f[p] += (R)cdir(p, d) * diff[d];
        }
    });
}

// Completion of one face cell; v = (ux, uy, uz) for velocity faces,
// (rho, -, -) for pressure faces.  FAM: 0 regularized velocity, 1 regularized
// pressure, 2 Zou/He velocity, 3 Zou/He pressure.
template <typename R, int FAM, int DIR, int ORI>
__device__ __forceinline__ void completeFaceT(R* f, const double* v) {
    R rhoBar, j[3];
    if (FAM == 0 || FAM == 2) {
        rhoBar = velFaceRhoBar<R, DIR, ORI>(f, (R)v[DIR]);
        R rho = rhoBar + (R)1;
#pragma unroll
        for (int d = 0; d < 3; ++d) j[d] = rho * ((R)v[d] - (R)0.5 * (R)0);
    } else {
        rhoBar = (R)v[0] - (R)1;
        pressFaceJ<R, DIR, ORI>(f, rhoBar, j);
    }
    if (FAM < 2) regularizedComplete<R, DIR, ORI>(f, rhoBar, j);
    else zouHeComplete<R, DIR, ORI>(f, rhoBar, j);
}

template <typename R, int FAM>
__device__ __forceinline__ void completeFaceFam(R* f, int sub, const double* v) {
    switch (sub) {
    case 0: completeFaceT<R, FAM, 0, -1>(f, v); break;
    case 1: completeFaceT<R, FAM, 0, 1>(f, v); break;
    case 2: completeFaceT<R, FAM, 1, -1>(f, v); break;
    case 3: completeFaceT<R, FAM, 1, 1>(f, v); break;
    case 4: completeFaceT<R, FAM, 2, -1>(f, v); break;
    default: completeFaceT<R, FAM, 2, 1>(f, v); break;
    }
}

template <typename R>
__device__ __noinline__ void completeFace(R* f, int kind, const double* v) {
    const int fam = faceFamily(kind), sub = (kind - K_REGVEL) % 6;
    switch (fam) {
    case 0: completeFaceFam<R, 0>(f, sub, v); break;
    case 1: completeFaceFam<R, 1>(f, sub, v); break;
    case 2: completeFaceFam<R, 2>(f, sub, v); break;
    default: completeFaceFam<R, 3>(f, sub, v); break;
    }
}

// Rho-bar of a velocity face cell (VelocityDirichletBoundaryDynamics::computeRhoBar)
// for a runtime direction / orientation.
template <typename R>
__device__ __noinline__ R velFaceRhoBarAny(const R* f, int kind, R velDir) {
    switch ((kind - K_REGVEL) % 6) {
    case 0: return velFaceRhoBar<R, 0, -1>(f, velDir);
    case 1: return velFaceRhoBar<R, 0, 1>(f, velDir);
    case 2: return velFaceRhoBar<R, 1, -1>(f, velDir);
    case 3: return velFaceRhoBar<R, 1, 1>(f, velDir);
    case 4: return velFaceRhoBar<R, 2, -1>(f, velDir);
    default: return velFaceRhoBar<R, 2, 1>(f, velDir);
    }
}

// Momentum of a pressure face cell (DensityDirichletBoundaryDynamics::computeJ)
// for a runtime direction / orientation.
template <typename R>
__device__ __noinline__ void pressFaceJAny(const R* f, int kind, R rhoBar, R* j) {
    switch ((kind - K_REGVEL) % 6) {
    case 0: pressFaceJ<R, 0, -1>(f, rhoBar, j); break;
    case 1: pressFaceJ<R, 0, 1>(f, rhoBar, j); break;
    case 2: pressFaceJ<R, 1, -1>(f, rhoBar, j); break;
    case 3: pressFaceJ<R, 1, 1>(f, rhoBar, j); break;
    case 4: pressFaceJ<R, 2, -1>(f, rhoBar, j); break;
    default: pressFaceJ<R, 2, 1>(f, rhoBar, j); break;
    }
}

}  // namespace plbgpu
