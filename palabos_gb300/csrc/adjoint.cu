// Discrete adjoint of the collide-and-stream step, with checkpointing, and a
// forward-mode (dual-number) tangent of the same step.  No counterpart in the
// reference: it differentiates the reference's step exactly as the fused
// kernels compute it.
//
// State: f-bar in natural (post-stream) order, structure of arrays, in the
// arithmetic type R (double for the FP64 form, float otherwise); plane i of
// state k lives at buf + (k * 19 + i) * n.  The step used here is a two-buffer
// push step with the same per-cell collision code as the fused kernels, so
// the FP64 trajectory is bit-identical to the domain's own.
//
// Objective: J = 1/2 sum over cells |u(T) - u*|^2, u the velocity each cell's
// dynamics reports (computeVelocity).  Dynamics: BGK, Guo-forced BGK,
// incompressible BGK, bounce-back, no-dynamics.
//
// Reverse step at cell x, given lambda^{n+1}:
//   mu_i(x)  = lambda^{n+1}_i(x + c_i), or lambda^{n+1}_opp(i)(x) where the
//              push step reflected the population (transpose of streaming);
//   lambda^n = (d collide / d f)^T mu at the pre-collision state f^n(x),
//              recomputed from the last checkpoint;
//   dJ/dF(x) += (d collide / d F)^T mu,   dJ/domega += (d collide / d omega)^T mu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <new>
#include <vector>

#include "../../include/plbgpu.h"
#include "launch.h"

namespace plbgpu {

// ---------------------------------------------------------------- dual numbers

template <typename T>
struct DualT {
    T v, d;
    __host__ __device__ DualT() : v(0), d(0) {}
    __host__ __device__ DualT(double x) : v((T)x), d(0) {}
    __host__ __device__ DualT(double x, double y) : v((T)x), d((T)y) {}
    __host__ __device__ DualT& operator+=(const DualT& o) { v += o.v; d += o.d; return *this; }
    __host__ __device__ DualT& operator-=(const DualT& o) { v -= o.v; d -= o.d; return *this; }
    __host__ __device__ DualT& operator*=(const DualT& o) { d = d * o.v + v * o.d; v *= o.v; return *this; }
};
template <typename T>
__host__ __device__ inline DualT<T> operator+(DualT<T> a, const DualT<T>& b) { return a += b; }
template <typename T>
__host__ __device__ inline DualT<T> operator-(DualT<T> a, const DualT<T>& b) { return a -= b; }
template <typename T>
__host__ __device__ inline DualT<T> operator*(DualT<T> a, const DualT<T>& b) { return a *= b; }
template <typename T>
__host__ __device__ inline DualT<T> operator-(const DualT<T>& a) { return DualT<T>(-a.v, -a.d); }
template <typename T>
__host__ __device__ inline DualT<T> operator/(const DualT<T>& a, const DualT<T>& b) {
    const T q = a.v / b.v;
    DualT<T> r;
    r.v = q;
    r.d = (a.d - q * b.d) / b.v;
    return r;
}
template <typename T>
__device__ inline DualT<T> invRhoOf(DualT<T> rhoBar) {
    const T r = (T)1 / (rhoBar.v + (T)1);
    DualT<T> out;
    out.v = r;
    out.d = -rhoBar.d * r * r;
    return out;
}
// FP64 duals (the tangent run, the FP64 adjoint) and FP32 duals (the FP32
// adjoint's face cells, on the FP32 pipe).
using Dual = DualT<double>;
using DualF = DualT<float>;
// The density of a dual rho-bar (the edge and corner processors' rounding to
// R has derivative one).
template <typename T>
__device__ inline DualT<T> densityOfRhoBar(DualT<T> rb) { return rb + DualT<T>(1.0); }

template <typename R> __device__ inline double valueOf(const R& x) { return (double)x; }
template <> __device__ inline double valueOf<Dual>(const Dual& x) { return x.v; }
template <typename R> __device__ inline double tangentOf(const R&) { return 0.; }
template <> __device__ inline double tangentOf<Dual>(const Dual& x) { return x.d; }

// ---------------------------------------------------------------- per-cell forward

template <typename R>
__device__ __forceinline__ void adjCollide(int k, R* f, const R* F, const BgkConst<R>& bc, R invRho0) {
    R rhoBar, j[3];
    if (bgkBase(k)) {   // BGK, and the BGK base of the face conditions
        rhoBarJ<R>(f, rhoBar, j);
        bgkCollide<R>(f, rhoBar, j, bc, invRhoOf(rhoBar));
        return;
    }
    switch (k) {
    case K_GUO: {
        R rb = rhoBarSeq<R>(f);
        R rb2, jj[3], u[3];
        rhoBarJ<R>(f, rb2, jj);
        R invRho = invRhoOf(rb2);
        for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho + F[d] / (R)2;
        R rho = rb + (R)1;
        for (int d = 0; d < 3; ++d) j[d] = rho * u[d];
        bgkCollide<R>(f, rb, j, bc, invRhoOf(rb));
        addGuoForce<R>(f, F, u, bc.omega);
        break;
    }
    case K_INCBGK:
        rhoBarJ<R>(f, rhoBar, j);
        bgkCollide<R>(f, rhoBar, j, bc, invRho0);
        break;
    case K_BB:
    case K_MEBB:   // bounce-back; the momentum it records is a side reduction
        for (int i = 1; i <= 9; ++i) {
            R t = f[i]; f[i] = f[i + 9]; f[i + 9] = t;
        }
        break;
    default:
        break;
    }
}

template <typename R>
__device__ __forceinline__ BgkConst<R> bgkConsts(R omega) {
    BgkConst<R> b;
    b.omega = omega;
    b.one_m_omega = (R)1 - omega;
    b.t0_omega = tw<R>(0) * omega;
    b.t1_omega = tw<R>(1) * omega;
    b.t4_omega = tw<R>(4) * omega;
    return b;
}

// The force planes are FP64 for FP64 (and dual) arithmetic, FP32 for FP32.
template <typename R>
__host__ __device__ constexpr bool forceIsFp64() { return sizeof(R) != sizeof(float); }

// Guo force of a cell: FP64 planes for the FP64 form, FP32 otherwise; `dF`
// (tangent runs only) gives its direction.
template <typename R>
__device__ __forceinline__ void cellForce(const DevLattice& L, bool fp64Force, long long idx, const double* dF, R* F) {
    for (int d = 0; d < 3; ++d) F[d] = R(0);
    if (L.force) {
        if (fp64Force) {
            const double* fp = static_cast<const double*>(L.force);
            for (int d = 0; d < 3; ++d) F[d] = R(fp[d * L.n + idx]);
        } else {
            const float* fp = static_cast<const float*>(L.force);
            for (int d = 0; d < 3; ++d) F[d] = R(fp[d * L.n + idx]);
        }
    }
}
__device__ __forceinline__ void cellForce(const DevLattice& L, bool fp64Force, long long idx, const double* dF,
                                          Dual* F) {
    double v[3] = {0., 0., 0.};
    if (L.force) {
        const double* fp = static_cast<const double*>(L.force);
        for (int d = 0; d < 3; ++d) v[d] = fp[d * L.n + idx];
    }
    for (int d = 0; d < 3; ++d) F[d] = Dual(v[d], dF ? dF[d * L.n + idx] : 0.);
}

// Velocity the way computeVelocity reports it (momentTemplates3D.h:402-408,
// externalForceDynamics.hh:58-73, isoThermalDynamics.hh:1388-1395); zero on
// walls and no-dynamics cells.
template <typename R>
__device__ __forceinline__ void cellVelocity(int k, const R* f, const R* F, R invRho0, R* u) {
    u[0] = u[1] = u[2] = R(0);
    if (k == K_BGK || k == K_GUO || k == K_INCBGK) {
        R rb, j[3];
        rhoBarJ<R>(f, rb, j);
        if (k == K_INCBGK) {
            for (int d = 0; d < 3; ++d) u[d] = j[d] * invRho0;
        } else {
            R invRho = invRhoOf(k == K_BGK ? rhoBarSeq<R>(f) : rb);
            for (int d = 0; d < 3; ++d) u[d] = j[d] * invRho + (k == K_GUO ? F[d] / (R)2 : R(0));
        }
    }
}

// ---------------------------------------------------------------- per-cell reverse

// lam = (d out / d f)^T mu for out = collide(f; F, omega); gF += (d out / d F)^T mu;
// returns (d out / d omega)^T mu.  BGK in shifted variables:
//   out_i = (1 - w) f_i + w feq_i(rhoBar, J) + a G_i,  a = 1 - w/2,
//   feq_i = t_i (rhoBar + 3 e_i + v (4.5 e_i^2 - 1.5 |J|^2)),  e_i = c_i.J,
//   v = 1/rho (1/rho0 for incompressible BGK),  rho = rhoBar + 1,
//   Guo: u = j/rho + F/2, J = rho u, G_i = t_i (3 (c_i - u).F + 9 (c_i.u)(c_i.F));
//   otherwise J = j, G = 0.
// Every sum over populations of mu_i times these terms is a contraction with
// the moments of nu_i = t_i mu_i: M0 = sum nu_i, M1 = sum nu_i c_i,
// M2 = sum nu_i c_i c_i^T, so the reverse pass costs about as much as the
// forward collision.
template <typename R>
__device__ R adjCell(int k, const R* f, const R* F, R omega, R invRho0, const R* mu, R* lam, R* gF) {
    if (k == K_BB || k == K_MEBB) {
        lam[0] = mu[0];
#pragma unroll
        for (int i = 1; i < 19; ++i) lam[i] = mu[opp(i)];
        return R(0);
    }
    if (k != K_BGK && k != K_GUO && k != K_INCBGK) {
#pragma unroll
        for (int i = 0; i < 19; ++i) lam[i] = mu[i];
        return R(0);
    }
    const bool guo = (k == K_GUO), inc = (k == K_INCBGK);
    // forward moments of f
    R rhoBar = R(0), j[3] = {R(0), R(0), R(0)}, muf = R(0);
    // moments of nu = t mu
    R M0 = R(0), M1[3] = {R(0), R(0), R(0)}, M2[6] = {R(0), R(0), R(0), R(0), R(0), R(0)};
#pragma unroll
    for (int i = 0; i < 19; ++i) {
        rhoBar += f[i];
        muf += mu[i] * f[i];
        const R nu = tw<R>(i) * mu[i];
        M0 += nu;
        const int cx = cdir(i, 0), cy = cdir(i, 1), cz = cdir(i, 2);
        if (cx) { j[0] += cx > 0 ? f[i] : -f[i]; M1[0] += cx > 0 ? nu : -nu; M2[0] += nu; }
        if (cy) { j[1] += cy > 0 ? f[i] : -f[i]; M1[1] += cy > 0 ? nu : -nu; M2[3] += nu; }
        if (cz) { j[2] += cz > 0 ? f[i] : -f[i]; M1[2] += cz > 0 ? nu : -nu; M2[5] += nu; }
        if (cx && cy) M2[1] += cx * cy > 0 ? nu : -nu;
        if (cx && cz) M2[2] += cx * cz > 0 ? nu : -nu;
        if (cy && cz) M2[4] += cy * cz > 0 ? nu : -nu;
    }
    // M2 packed as xx, xy, xz, yy, yz, zz
    auto m2v = [&](const R* a, R* out) {
        out[0] = M2[0] * a[0] + M2[1] * a[1] + M2[2] * a[2];
        out[1] = M2[1] * a[0] + M2[3] * a[1] + M2[4] * a[2];
        out[2] = M2[2] * a[0] + M2[4] * a[1] + M2[5] * a[2];
    };
    const R rho = rhoBar + (R)1;
    const R invRho = (R)1 / rho;
    R u[3], Jp[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        u[d] = j[d] * invRho + (guo ? F[d] / (R)2 : R(0));
        Jp[d] = guo ? rho * u[d] : j[d];
    }
    const R v = inc ? invRho0 : invRho;
    const R Q = Jp[0] * Jp[0] + Jp[1] * Jp[1] + Jp[2] * Jp[2];
    R M2J[3];
    m2v(Jp, M2J);
    const R JM2J = Jp[0] * M2J[0] + Jp[1] * M2J[1] + Jp[2] * M2J[2];
    const R M1J = M1[0] * Jp[0] + M1[1] * Jp[1] + M1[2] * Jp[2];
    // feq part
    const R sumMuFeq = rhoBar * M0 + (R)3 * M1J + v * ((R)4.5 * JM2J - (R)1.5 * Q * M0);
    const R QBar = -(R)1.5 * omega * v * M0;
    const R vBar = omega * ((R)4.5 * JM2J - (R)1.5 * Q * M0);
    R JBar[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) JBar[d] = omega * ((R)3 * M1[d] + (R)9 * v * M2J[d]) + (R)2 * QBar * Jp[d];
    R rhoBarBar = omega * M0 + (inc ? R(0) : -v * v * vBar);
    R jBar[3] = {JBar[0], JBar[1], JBar[2]};
    R sumMuG = R(0);
    if (guo) {
        const R a = (R)1 - omega / (R)2;
        R M2F[3], M2u[3];
        m2v(F, M2F);
        m2v(u, M2u);
        const R uF = u[0] * F[0] + u[1] * F[1] + u[2] * F[2];
        const R M1F = M1[0] * F[0] + M1[1] * F[1] + M1[2] * F[2];
        const R uM2F = u[0] * M2F[0] + u[1] * M2F[1] + u[2] * M2F[2];
        sumMuG = (R)3 * M1F - (R)3 * uF * M0 + (R)9 * uM2F;
        R uBar[3], FBar[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            uBar[d] = a * (-(R)3 * M0 * F[d] + (R)9 * M2F[d]);
            FBar[d] = a * ((R)3 * M1[d] - (R)3 * M0 * u[d] + (R)9 * M2u[d]);
        }
        // J = j + (rho/2) F
        rhoBarBar += (F[0] * JBar[0] + F[1] * JBar[1] + F[2] * JBar[2]) / (R)2;
        // u = j / rho + F / 2
        const R ju = j[0] * uBar[0] + j[1] * uBar[1] + j[2] * uBar[2];
        rhoBarBar += -ju * invRho * invRho;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            FBar[d] += rho / (R)2 * JBar[d] + uBar[d] / (R)2;
            jBar[d] += uBar[d] * invRho;
            gF[d] += FBar[d];
        }
    }
    const R om1 = (R)1 - omega;
#pragma unroll
    for (int i = 0; i < 19; ++i) {
        R l = om1 * mu[i] + rhoBarBar;
        const int cx = cdir(i, 0), cy = cdir(i, 1), cz = cdir(i, 2);
        if (cx) l += cx > 0 ? jBar[0] : -jBar[0];
        if (cy) l += cy > 0 ? jBar[1] : -jBar[1];
        if (cz) l += cz > 0 ? jBar[2] : -jBar[2];
        lam[i] = l;
    }
    return sumMuFeq - muf - sumMuG / (R)2;
}

// ---------------------------------------------------------------- kernels

// Neighbour of a cell along +c_i.  INTERIOR rows (1 <= x <= nx-2,
// 1 <= y <= ny-2) use the uniform offsets c_i . (ny*nz, nz, 1) and only check
// the z ends; border rows use the general neighbourhood.  Returns false where
// a non-periodic domain is left.  A block covers part of one row, so the
// kernels pick the form once per block.
template <bool INTERIOR>
struct CellMoves;

template <>
struct CellMoves<true> {
    long long wrapM, wrapP;
    bool okM, okP;
    __device__ __forceinline__ CellMoves(const DevLattice& L, int, int, int z) {
        wrapM = z == 0 ? L.nz : 0;
        wrapP = z == L.nz - 1 ? -L.nz : 0;
        okM = z > 0 || L.per[2];
        okP = z < L.nz - 1 || L.per[2];
    }
    __device__ __forceinline__ bool plus(int i, const int* D, long long& off) const {
        const int cz = cdir(i, 2);
        off = D[i] + (cz < 0 ? wrapM : cz > 0 ? wrapP : 0);
        return cz < 0 ? okM : cz > 0 ? okP : true;
    }
};

template <>
struct CellMoves<false> {
    Neighbourhood nb;
    __device__ __forceinline__ CellMoves(const DevLattice& L, int x, int y, int z) : nb(neighbourhood(L, x, y, z)) {}
    __device__ __forceinline__ bool plus(int i, const int*, long long& off) const { return nb.move(i, +1, off); }
};

__device__ __forceinline__ bool interiorRow(const DevLattice& L, int x, int y) {
    return x > 0 && x < L.nx - 1 && y > 0 && y < L.ny - 1;
}

struct NeighbourDeltas {
    int d[19];
};

inline NeighbourDeltas deltasOf(const DevLattice& L) {
    NeighbourDeltas D;
    for (int i = 0; i < 19; ++i) D.d[i] = cdir(i, 0) * L.ny * L.nz + cdir(i, 1) * L.nz + cdir(i, 2);
    return D;
}

// Sums of the backward sweep, kept in kAdjSlots copies (one per block index
// modulo kAdjSlots) and added up on the host: one address taking an atomic
// from every warp of every step would serialize the sweep.
constexpr int kAdjSlots = 64;

struct AdjAcc {
    double objective[kAdjSlots];
    double gOmega[kAdjSlots];
    double tangent[kAdjSlots];
};

inline double slotSum(const double* v) {
    double s = 0.;
    for (int i = 0; i < kAdjSlots; ++i) s += v[i];
    return s;
}

// Block-wide sum of v, one atomic per block on its slot of dst.  Every thread
// of the block calls it.
__device__ __forceinline__ void blockAdd(double v, double* dst) {
    __shared__ double part[32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
    __syncthreads();   // part may still be read by a previous call
    if (lane == 0) part[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < nw ? part[lane] : 0.;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        const unsigned b = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
        if (lane == 0 && v != 0.) atomicAdd(dst + (b & (kAdjSlots - 1)), v);
    }
}

// Natural-order copy of the domain's state (either AA parity) and back.
template <typename S, typename R, bool ODD>
__global__ void stateOutKernel(DevLattice L, R* out) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    if (z >= L.nz) return;
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    Neighbourhood nb = neighbourhood(L, x, y, z);
    const S* P = static_cast<const S*>(L.pop);
    for (int i = 0; i < 19; ++i) out[i * L.n + idx] = R(StoreT<S>::ld(P + slotOf<ODD>(L, nb, idx, i)));
}

template <typename S, typename R>
__global__ void stateInKernel(DevLattice L, const R* in) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    if (z >= L.nz) return;
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    S* P = static_cast<S*>(L.pop);
    for (int i = 0; i < 19; ++i) StoreT<S>::st(P + i * L.stride + idx, (typename StoreT<S>::R)in[i * L.n + idx]);
}

// Push step fin -> fout (natural order): collide, then send f*_i to x + c_i
// or, leaving a non-periodic domain, back into slot opp(i) of x.
template <typename R, bool INTERIOR>
__device__ __forceinline__ void pushCell(const DevLattice& L, const NeighbourDeltas& D, const R* fin, R* fout,
                                         R omega, R invRho0, const double* dF, bool pending, int x, int y, int z) {
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    const int k = L.flags[idx];
    R f[19], F[3];
    for (int i = 0; i < 19; ++i) f[i] = fin[i * L.n + idx];
    // a face cell's missing populations are completed before it collides
    // when the state comes from a streaming step, as in the fused step
    if (pending && isFace(k)) completeIfFace<R>(L, idx, k, f);
    cellForce(L, forceIsFp64<R>(), idx, dF, F);
    adjCollide<R>(k, f, F, bgkConsts<R>(omega), invRho0);
    CellMoves<INTERIOR> mv(L, x, y, z);
    fout[idx] = f[0];
#pragma unroll
    for (int i = 1; i < 19; ++i) {
        long long off;
        fout[mv.plus(i, D.d, off) ? i * L.n + idx + off : opp(i) * L.n + idx] = f[i];
    }
}

template <typename R>
__global__ void pushStepKernel(DevLattice L, NeighbourDeltas D, const R* fin, R* fout, R omega, R invRho0,
                               const double* dF, bool pending) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    if (z >= L.nz) return;
    if (interiorRow(L, x, y)) pushCell<R, true>(L, D, fin, fout, omega, invRho0, dF, pending, x, y, z);
    else pushCell<R, false>(L, D, fin, fout, omega, invRho0, dF, pending, x, y, z);
}

// J, lambda^T = dJ/df^T and the explicit dJ/dF of the Guo velocity u = j/rho + F/2.
// Two objectives: the mismatch J = 1/2 sum |u - u*|^2 (v = u*), and the
// weighted velocity J = sum w . u (v = w, `weighted`), e.g. the mean flux.
template <typename R>
__global__ void objectiveKernel(DevLattice L, const R* f, const double* v, bool weighted, R invRho0, R* lam,
                                R* gF, AdjAcc* acc) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    double jsum = 0.;
    if (z < L.nz) {
        const long long idx = ((long long)x * L.ny + y) * L.nz + z;
        const int k = L.flags[idx];
        R fc[19], F[3], u[3];
        for (int i = 0; i < 19; ++i) fc[i] = f[i * L.n + idx];
        cellForce(L, forceIsFp64<R>(), idx, nullptr, F);
        cellVelocity<R>(k, fc, F, invRho0, u);
        R dv[3];   // dJ/du
        for (int d = 0; d < 3; ++d) {
            if (weighted) {
                dv[d] = (R)v[3 * idx + d];
                jsum += v[3 * idx + d] * (double)u[d];
            } else {
                dv[d] = u[d] - (R)v[3 * idx + d];
                jsum += 0.5 * (double)dv[d] * (double)dv[d];
            }
        }
        if (k == K_BGK || k == K_GUO || k == K_INCBGK) {
            R rho = R(1), jv[3] = {R(0), R(0), R(0)};
            for (int i = 0; i < 19; ++i) {
                rho += fc[i];
                for (int d = 0; d < 3; ++d) jv[d] += (R)cdir(i, d) * fc[i];
            }
            const R s = (k == K_INCBGK) ? invRho0 : (R)1 / rho;
            const R dj = (k == K_INCBGK) ? R(0) : (dv[0] * jv[0] + dv[1] * jv[1] + dv[2] * jv[2]) * s;
            for (int i = 0; i < 19; ++i)
                lam[i * L.n + idx] = ((R)cdir(i, 0) * dv[0] + (R)cdir(i, 1) * dv[1] + (R)cdir(i, 2) * dv[2] - dj) * s;
            if (k == K_GUO)
                for (int d = 0; d < 3; ++d) gF[d * L.n + idx] += dv[d] / (R)2;
        } else {
            for (int i = 0; i < 19; ++i) lam[i * L.n + idx] = R(0);
        }
    }
    blockAdd(jsum, acc->objective);
}

// Reverse of a face cell's completion: lam = (d complete / d f)^T nu for the
// wrapped regularized or Zou/He velocity or pressure condition of direction
// DIR and orientation ORI (the forward map is completeFaceT of d3q19.cuh:
// velFaceRhoBar / pressFaceJ, then regularizedComplete or zouHeComplete), in
// exact arithmetic.  f is the streamed state before completion, v the face's
// stored velocity (or density in v[0]).  The populations that enter from
// outside (c[DIR] = -ORI) are overwritten unread: their entries of lam are 0.
//
// Forward, with w_i = 1 on c[DIR] = 0 and 2 on c[DIR] = ORI (the known
// populations), e_i = c_i.j:
//   velocity face: rhoBar = (sum_i w_i f_i - u_n) / (1 + u_n), j = (rhoBar + 1) u;
//   pressure face: rhoBar = rho - 1,  j_DIR = ORI (sum_i w_i f_i - rhoBar);
//   feq_i = t_i (rhoBar + 3 e_i + (4.5 e_i^2 - 1.5 j.j) / (rhoBar + 1));
//   regularized: Pi = sum_known w_i c_i c_i^T (f_i - feq_i),
//                out_i = feq_i + 4.5 t_i (c_i c_i^T - I/3) : Pi;
//   Zou/He: f'_p = f_opp(p) - feq_opp(p) + feq_p on the incoming p, then the
//           incoming diagonals p get c_p,d (j_d - sum_i c_i,d f'_i) / nd along
//           the two tangential axes d.
template <typename R, int FAM, int DIR, int ORI>
__device__ __forceinline__ void completeFaceAdjT(const R* f, const double* v, const R* nu, R* lam) {
    // the forward quantities the reverse needs
    R rhoBar, j[3];
    const R vel[3] = {(R)v[0], (R)v[1], (R)v[2]};
    const R velNormal = (R)ORI * vel[DIR];
    if (FAM == 0 || FAM == 2) {
        rhoBar = velFaceRhoBar<R, DIR, ORI>(f, vel[DIR]);
        const R rho = rhoBar + (R)1;
#pragma unroll
        for (int d = 0; d < 3; ++d) j[d] = rho * vel[d];
    } else {
        rhoBar = (R)v[0] - (R)1;
        pressFaceJ<R, DIR, ORI>(f, rhoBar, j);
    }
    const R invRho = (R)1 / (rhoBar + (R)1);
    const R jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    R feqW[19];   // adjoint weight of each feq_i
#pragma unroll
    for (int i = 0; i < 19; ++i) {
        lam[i] = R(0);
        feqW[i] = R(0);
    }
    if (FAM < 2) {   // regularized
        R nuPi[6];
        int iPi = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = a; b < 3; ++b) {
                R s = R(0);
#pragma unroll
                for (int i = 0; i < 19; ++i) {
                    const R q = a == b ? (R)(cdir(i, a) * cdir(i, a)) - (R)1 / (R)3 : (R)2 * (R)(cdir(i, a) * cdir(i, b));
                    s += nu[i] * tw<R>(i) * q;
                }
                nuPi[iPi++] = (R)4.5 * s;
            }
#pragma unroll
        for (int i = 0; i < 19; ++i) {
            const int c = cdir(i, DIR);
            R nuFneq = R(0);
            if (c == 0 || c == ORI) {
                iPi = 0;
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int b = a; b < 3; ++b) nuFneq += (R)(cdir(i, a) * cdir(i, b)) * nuPi[iPi++];
                nuFneq *= (c == 0) ? (R)1 : (R)2;
                lam[i] += nuFneq;
            }
            feqW[i] = nu[i] - nuFneq;
        }
    } else {         // Zou/He
        constexpr int nd = subIndexCount<DIR, ORI>() - 1;
        R nuP[19];
#pragma unroll
        for (int i = 0; i < 19; ++i) nuP[i] = nu[i];
        R nuDiff[3] = {R(0), R(0), R(0)};
        forEachZh<DIR, ORI, true>([&](auto p) {
#pragma unroll
            for (int s2 = 1; s2 < 3; ++s2) {
                const int d = (DIR + s2) % 3;
                nuDiff[d] += (R)cdir(p, d) * nu[p];
            }
        });
        R jBarT[3] = {R(0), R(0), R(0)};
#pragma unroll
        for (int s2 = 1; s2 < 3; ++s2) {
            const int d = (DIR + s2) % 3;
            jBarT[d] = nuDiff[d] / (R)nd;
#pragma unroll
            for (int i = 0; i < 19; ++i) nuP[i] -= (R)cdir(i, d) * jBarT[d];
        }
        bool missing[19];
#pragma unroll
        for (int i = 0; i < 19; ++i) missing[i] = false;
        forEachZh<DIR, ORI, false>([&](auto p) {
            missing[p] = true;
            const int o = opp(p);
            lam[o] += nuP[p];
            feqW[o] -= nuP[p];
            feqW[p] += nuP[p];
        });
#pragma unroll
        for (int i = 0; i < 19; ++i)
            if (!missing[i]) lam[i] += nuP[i];
        // the face's own j enters the tangential correction directly
        if (FAM == 2) {
            R rbT = R(0);
#pragma unroll
            for (int d = 0; d < 3; ++d) rbT += jBarT[d] * vel[d];
            const R s = rbT / ((R)1 + velNormal);
#pragma unroll
            for (int i = 0; i < 19; ++i) {
                const int c = cdir(i, DIR);
                if (c == 0) lam[i] += s;
                else if (c == ORI) lam[i] += (R)2 * s;
            }
        }
    }
    // through feq_i(rhoBar, j)
    R rbBar = R(0), jBar[3] = {R(0), R(0), R(0)};
#pragma unroll
    for (int i = 0; i < 19; ++i) {
        const R e = (R)cdir(i, 0) * j[0] + (R)cdir(i, 1) * j[1] + (R)cdir(i, 2) * j[2];
        const R w = feqW[i] * tw<R>(i);
        rbBar += w * ((R)1 - invRho * invRho * ((R)4.5 * e * e - (R)1.5 * jSqr));
#pragma unroll
        for (int d = 0; d < 3; ++d) jBar[d] += w * ((R)3 * (R)cdir(i, d) + invRho * ((R)9 * e * (R)cdir(i, d) - (R)3 * j[d]));
    }
    // through (rhoBar, j) to the known populations
    if (FAM == 0 || FAM == 2) {
#pragma unroll
        for (int d = 0; d < 3; ++d) rbBar += jBar[d] * vel[d];
        const R s = rbBar / ((R)1 + velNormal);
#pragma unroll
        for (int i = 0; i < 19; ++i) {
            const int c = cdir(i, DIR);
            if (c == 0) lam[i] += s;
            else if (c == ORI) lam[i] += (R)2 * s;
        }
    } else {
        const R s = (R)ORI * jBar[DIR];
#pragma unroll
        for (int i = 0; i < 19; ++i) {
            const int c = cdir(i, DIR);
            if (c == 0) lam[i] += s;
            else if (c == ORI) lam[i] += (R)2 * s;
        }
    }
}

template <typename R, int FAM>
__device__ __forceinline__ void completeFaceAdjFam(int sub, const R* f, const double* v, const R* nu, R* lam) {
    switch (sub) {
    case 0: completeFaceAdjT<R, FAM, 0, -1>(f, v, nu, lam); break;
    case 1: completeFaceAdjT<R, FAM, 0, 1>(f, v, nu, lam); break;
    case 2: completeFaceAdjT<R, FAM, 1, -1>(f, v, nu, lam); break;
    case 3: completeFaceAdjT<R, FAM, 1, 1>(f, v, nu, lam); break;
    case 4: completeFaceAdjT<R, FAM, 2, -1>(f, v, nu, lam); break;
    default: completeFaceAdjT<R, FAM, 2, 1>(f, v, nu, lam); break;
    }
}

template <typename R>
__device__ __noinline__ void completeFaceAdj(int kind, const R* f, const double* v, const R* nu, R* lam) {
    const int fam = (kind - K_REGVEL) / 6, sub = (kind - K_REGVEL) % 6;
    switch (fam) {
    case 0: completeFaceAdjFam<R, 0>(sub, f, v, nu, lam); break;
    case 1: completeFaceAdjFam<R, 1>(sub, f, v, nu, lam); break;
    case 2: completeFaceAdjFam<R, 2>(sub, f, v, nu, lam); break;
    default: completeFaceAdjFam<R, 3>(sub, f, v, nu, lam); break;
    }
}

// Reverse step of the face cells (regularized and Zou/He velocity and
// pressure faces), one thread per cell of `faces`: the cell's local map is
// out = collide(complete(f)) (completion only when `pending`, collision with
// the BGK base), so lambda^n = (d complete / d f)^T (d collide / d g)^T mu
// with g = complete(f): the BGK reverse of adjCell on the completed state,
// then the closed-form reverse of the completion.  The omega derivative is
// the collision's.
template <typename R>
__global__ void faceAdjointKernel(DevLattice L, const R* f, const R* lamIn, R* lamOut, double omega, bool pending,
                                  const long long* faces, int nFaces, AdjAcc* acc) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double go = 0.;
    if (t < nFaces) {
        const long long idx = faces[t];
        const int z = (int)(idx % L.nz), y = (int)((idx / L.nz) % L.ny), x = (int)(idx / ((long long)L.ny * L.nz));
        const int k = L.flags[idx];
        const Neighbourhood nb = neighbourhood(L, x, y, z);
        R mu[19], fc[19], g[19], nu[19], F[3] = {R(0), R(0), R(0)}, gF[3] = {R(0), R(0), R(0)};
        mu[0] = lamIn[idx];
        for (int i = 1; i < 19; ++i) {
            long long off;
            mu[i] = nb.move(i, +1, off) ? lamIn[i * L.n + idx + off] : lamIn[opp(i) * L.n + idx];
        }
        for (int i = 0; i < 19; ++i) fc[i] = g[i] = f[i * L.n + idx];
        if (pending) completeIfFace<R>(L, idx, k, g);
        go = (double)adjCell<R>(K_BGK, g, F, (R)omega, R(0), mu, nu, gF);
        if (pending) {
            const double v[3] = {L.bc[idx], L.bc[L.n + idx], L.bc[2 * L.n + idx]};
            R lam[19];
            completeFaceAdj<R>(k, fc, v, nu, lam);
            for (int i = 0; i < 19; ++i) lamOut[i * L.n + idx] = lam[i];
        } else {
            for (int i = 0; i < 19; ++i) lamOut[i * L.n + idx] = nu[i];
        }
    }
    blockAdd(go, acc->gOmega);
}

// Drag objective J = w . D(f) with D the momentum-exchange drag the next
// collision records (bounceBackModels.hh:100-136): over the fluid directions i
// of each momentum-exchange cell, D -= 2 c_i f_opp(i).  Linear in f, so
// lambda is -2 w . c_i on population opp(i) of those cells and zero elsewhere;
// no explicit force term.
template <typename R>
__global__ void dragObjectiveKernel(DevLattice L, const R* f, double w0, double w1, double w2, R* lam, AdjAcc* acc) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    double jsum = 0.;
    if (z < L.nz) {
        const long long idx = ((long long)x * L.ny + y) * L.nz + z;
        const uint32_t mask = L.flags[idx] == K_MEBB ? L.mebb[idx] : 0u;
        R l[19];
        for (int i = 0; i < 19; ++i) l[i] = R(0);
#pragma unroll
        for (int i = 1; i < 19; ++i) {
            if (!(mask & (1u << i))) continue;
            const double c = -2. * (w0 * cdir(i, 0) + w1 * cdir(i, 1) + w2 * cdir(i, 2));
            l[opp(i)] += (R)c;
            jsum += c * (double)f[opp(i) * L.n + idx];
        }
        for (int i = 0; i < 19; ++i) lam[i * L.n + idx] = l[i];
    }
    blockAdd(jsum, acc->objective);
}

__global__ void dualDragObjectiveKernel(DevLattice L, const Dual* f, double w0, double w1, double w2,
                                        AdjAcc* acc) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    double jv = 0., jd = 0.;
    if (z < L.nz) {
        const long long idx = ((long long)x * L.ny + y) * L.nz + z;
        const uint32_t mask = L.flags[idx] == K_MEBB ? L.mebb[idx] : 0u;
        for (int i = 1; i < 19; ++i) {
            if (!(mask & (1u << i))) continue;
            const double c = -2. * (w0 * cdir(i, 0) + w1 * cdir(i, 1) + w2 * cdir(i, 2));
            const Dual fo = f[opp(i) * L.n + idx];
            jv += c * fo.v;
            jd += c * fo.d;
        }
    }
    blockAdd(jv, acc->objective);
    blockAdd(jd, acc->tangent);
}

// One reverse step: lamIn = lambda^{n+1}, f = f^n (pre-collision), lamOut = lambda^n.
template <typename R, bool INTERIOR>
__device__ __forceinline__ R adjointCell(const DevLattice& L, const NeighbourDeltas& D, const R* f, const R* lamIn,
                                         R* lamOut, R* gF, R omega, R invRho0, int x, int y, int z) {
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    const int k = L.flags[idx];
    if (isFace(k)) return R(0);   // faceAdjointKernel reverses the face cells
    CellMoves<INTERIOR> mv(L, x, y, z);
    R mu[19], fc[19], F[3], lam[19], g[3] = {R(0), R(0), R(0)};
    mu[0] = lamIn[idx];
#pragma unroll
    for (int i = 1; i < 19; ++i) {
        long long off;
        mu[i] = lamIn[mv.plus(i, D.d, off) ? i * L.n + idx + off : opp(i) * L.n + idx];
    }
    for (int i = 0; i < 19; ++i) fc[i] = f[i * L.n + idx];
    cellForce(L, forceIsFp64<R>(), idx, nullptr, F);
    // an edge or corner cell collides with its BGK base
    const R go = adjCell<R>(isSurface(k) ? K_BGK : k, fc, F, omega, invRho0, mu, lam, g);
    for (int i = 0; i < 19; ++i) lamOut[i * L.n + idx] = lam[i];
    if (k == K_GUO)
        for (int d = 0; d < 3; ++d) gF[d * L.n + idx] += g[d];
    return go;
}

template <typename R>
__global__ void adjointStepKernel(DevLattice L, NeighbourDeltas D, const R* f, const R* lamIn, R* lamOut, R* gF,
                                  R omega, R invRho0, AdjAcc* acc) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    double go = 0.;
    if (z < L.nz) {
        go = interiorRow(L, x, y) ? (double)adjointCell<R, true>(L, D, f, lamIn, lamOut, gF, omega, invRho0, x, y, z)
                                  : (double)adjointCell<R, false>(L, D, f, lamIn, lamOut, gF, omega, invRho0, x, y, z);
    }
    blockAdd(go, acc->gOmega);
}

// J and its tangent from a dual state.
__global__ void dualObjectiveKernel(DevLattice L, const Dual* f, const double* dF, const double* v, bool weighted,
                                    double invRho0, AdjAcc* acc) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    double jv = 0., jd = 0.;
    if (z < L.nz) {
        const long long idx = ((long long)x * L.ny + y) * L.nz + z;
        const int k = L.flags[idx];
        Dual fc[19], F[3], u[3];
        for (int i = 0; i < 19; ++i) fc[i] = f[i * L.n + idx];
        cellForce(L, true, idx, dF, F);
        cellVelocity<Dual>(k, fc, F, Dual(invRho0), u);
        for (int d = 0; d < 3; ++d) {
            if (weighted) {
                jv += v[3 * idx + d] * u[d].v;
                jd += v[3 * idx + d] * u[d].d;
            } else {
                const Dual dv = u[d] - Dual(v[3 * idx + d]);
                jv += 0.5 * dv.v * dv.v;
                jd += dv.v * dv.d;
            }
        }
    }
    blockAdd(jv, acc->objective);
    blockAdd(jd, acc->tangent);
}

template <typename R>
__global__ void toDualKernel(long long n19, const double* in, Dual* out) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n19) out[i] = Dual(in[i], 0.);
}

// ---------------------------------------------------------------- edges and corners
//
// The external velocity edges and corners (finite-difference processors) run
// after each push step, edges first, then corners, on the natural-order state:
// the same arithmetic as the domain's own surfaceKernel (kernels.cuh), in the
// adjoint's arithmetic T (R, or a dual number for the tangent run).

// Populations of a natural-order state.
template <typename T>
struct NatSource {
    const T* buf;
    long long n;
    __device__ __forceinline__ void operator()(int, int, int, long long idx, T* f) const {
#pragma unroll
        for (int i = 0; i < 19; ++i) f[i] = buf[i * n + idx];
    }
};

template <typename R, typename T>
__global__ void surfaceNatKernel(DevLattice L, T* buf, const int4* cells, int count, R invRho0, double bbRho,
                                 T omega) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int4 c = cells[t];
    const long long idx = ((long long)c.x * L.ny + c.y) * L.nz + c.z;
    NatSource<T> src{buf, L.n};
    T rho, g[3][3], vel[3], f[19];
    // after a push step the faces are as streamed: their completion is pending
    surfaceGradients<R, T>(L, c, 1, invRho0, bbRho, src, rho, g);
#pragma unroll
    for (int d = 0; d < 3; ++d) vel[d] = T((R)L.bc[d * L.n + idx]);
    surfaceFromGradients<T>(rho, g, vel, omega, f);
    for (int i = 0; i < 19; ++i) buf[i * L.n + idx] = f[i];
}

// Populations of a natural-order state as dual numbers, with the derivative
// seeded on population `pop` of cell `seed`.
template <typename R>
struct SeededSource {
    const R* buf;
    long long n, seed;
    int pop;
    __device__ __forceinline__ void operator()(int, int, int, long long idx, DualT<R>* f) const {
#pragma unroll
        for (int i = 0; i < 19; ++i) f[i] = DualT<R>(buf[i * n + idx], (idx == seed && i == pop) ? 1.0 : 0.0);
    }
};

// The cells an edge or corner processor reads that carry a derivative:
// candidate r of cell c (the inward neighbours, then for an edge the two
// along it).  Returns the cell index, or -1 when candidate r reads nothing
// differentiable (a wall, a cell outside the lattice, or a cell that stores
// its velocity read for its velocity only).
__device__ __forceinline__ long long surfaceCandidate(const DevLattice& L, int4 c, int r) {
    const bool edge = c.w < K_CORNER;
    int axis, side;
    bool velocityOnly = false;
    if (edge) {
        const int e = c.w - K_EDGE, plane = e / 4;
        if (r == 0) { axis = (plane + 1) % 3; side = (e & 2) ? -1 : 1; }
        else if (r == 1) { axis = (plane + 2) % 3; side = (e & 1) ? -1 : 1; }
        else { axis = plane; side = r == 2 ? 1 : -1; velocityOnly = true; }
    } else {
        const int q = c.w - K_CORNER;
        axis = r;
        side = (q & (4 >> r)) ? -1 : 1;
    }
    int p[3] = {c.x, c.y, c.z};
    p[axis] += side;
    const long long qi = ((long long)wrapAxis(p[0], L.nx) * L.ny + wrapAxis(p[1], L.ny)) * L.nz + wrapAxis(p[2], L.nz);
    const int k = L.flags[qi];
    if (k == K_BB || k == K_MEBB || k == K_NODYN || k == K_NONE) return -1;
    if (velocityOnly && (isSurface(k) || (isFace(k) && (faceFamily(k) == 0 || faceFamily(k) == 2)))) return -1;
    return qi;
}

// Number of dual passes of one edge (corner) cell: omega, then 19 per candidate.
__host__ __device__ constexpr int surfacePasses(bool edge) { return 1 + 19 * (edge ? 4 : 3); }

// Reverse of the edge (or corner) processor of one launch's cells on lambda,
// at the state f it produced, one dual pass per thread: pass 0 of a cell
// gives the omega derivative (to gOmega), pass 1 + 19 r + j the derivative
// with respect to population j of the cell's candidate r -- the whole
// processor (finite differences, face completion of a pending neighbour,
// rebuild) differentiated at once -- contracted with the cell's 19 adjoint
// values and added to that population's.  The cell's own incoming
// populations, overwritten unread, get zero afterwards (surfaceAdjointZero).
// Corners read edges' densities, so the corners' reverse runs first.
template <typename R>
__global__ void surfaceAdjointKernel(DevLattice L, const R* f, R* lam, const int4* cells, int count, int passes,
                                     R invRho0, double bbRho, R omega, AdjAcc* acc) {
    using D = DualT<R>;
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double go = 0.;
    if (g < (long long)count * passes) {
        const int t = (int)(g / passes), pass = (int)(g - (long long)t * passes);
        const int4 c = cells[t];
        const long long idx = ((long long)c.x * L.ny + c.y) * L.nz + c.z;
        const long long qi = pass == 0 ? -1 : surfaceCandidate(L, c, (pass - 1) / 19);
        if (pass == 0 || qi >= 0) {
            const int j = pass == 0 ? 0 : (pass - 1) % 19;
            SeededSource<R> src{f, L.n, qi, j};
            D rho, gr[3][3], vel[3], fo[19];
            surfaceGradients<R, D>(L, c, 1, invRho0, bbRho, src, rho, gr);
            for (int d = 0; d < 3; ++d) vel[d] = D((R)L.bc[d * L.n + idx]);
            surfaceFromGradients<D>(rho, gr, vel, D(omega, pass == 0 ? 1.0 : 0.0), fo);
            R v = R(0);
            for (int i = 0; i < 19; ++i) v += lam[i * L.n + idx] * fo[i].d;
            if (pass == 0) go = (double)v;
            else if (v != R(0)) atomicAdd(&lam[j * L.n + qi], v);
        }
    }
    blockAdd(go, acc->gOmega);
}

// The edge and corner cells' own adjoint values, once their reverse has read them.
template <typename R>
__global__ void surfaceAdjointZero(DevLattice L, R* lam, const int4* cells, int count) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const int4 c = cells[t];
    const long long idx = ((long long)c.x * L.ny + c.y) * L.nz + c.z;
    for (int i = 0; i < 19; ++i) lam[i * L.n + idx] = R(0);
}

// ---------------------------------------------------------------- host side

namespace {

struct AdjointState {
    int precision = -1;
    long long n = 0;
    int T = 0, K = 0, nckpt = 0;
    void* ckpt = nullptr;      // (nckpt) states
    void* seg = nullptr;       // (K + 1) states
    void* seg2 = nullptr;      // a second segment, recomputed beside the reverse of the first (or null)
    cudaStream_t side = nullptr;   // the stream that recomputes the next segment
    cudaEvent_t fork = nullptr, join = nullptr;
    void* lam = nullptr;       // 2 states
    void* gF = nullptr;        // 3 planes
    double* uT = nullptr;      // target velocity, n * 3
    AdjAcc* acc = nullptr;
    long long* faces = nullptr;   // face cells (cell indices), nFaces of them
    int nFaces = 0;
    int4* surf = nullptr;         // edge cells, then corner cells (x, y, z, kind)
    int nEdges = 0, nCorners = 0;
    bool pending0 = false;     // the recorded run's first step completes its faces
    bool ready = false;        // a forward run is recorded
    ~AdjointState() {
        cudaFree(ckpt); cudaFree(seg); cudaFree(lam); cudaFree(gF); cudaFree(uT); cudaFree(acc); cudaFree(faces);
        cudaFree(surf); cudaFree(seg2);
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (side) cudaStreamDestroy(side);
    }
    // Steps after the first collide states that came from a streaming step:
    // their faces are completed first.
    bool pendingAt(long long t) const { return t == 0 ? pending0 : nFaces > 0; }
};

void freeAdjoint(void* p) { delete static_cast<AdjointState*>(p); }

// One thread per cell, a block per row segment; short rows get fewer threads.
int cellBlock(const DevLattice& L) {
    const int t = (L.nz + 31) / 32 * 32;
    return t < 128 ? t : 128;
}
dim3 cellGrid(const DevLattice& L) { return rowGrid(L.nz, L.ny, L.nx, cellBlock(L)); }

template <typename S, typename R>
void stateOut(const DevLattice& L, bool odd, R* out, cudaStream_t s) {
    if (odd) stateOutKernel<S, R, true><<<cellGrid(L), cellBlock(L), 0, s>>>(L, out);
    else stateOutKernel<S, R, false><<<cellGrid(L), cellBlock(L), 0, s>>>(L, out);
}

template <typename R>
void stateOutAny(int prec, const DevLattice& L, bool odd, R* out, cudaStream_t s) {
    switch (prec) {
    case PLBGPU_FP64: stateOut<double, R>(L, odd, out, s); break;
    case PLBGPU_FP32: stateOut<float, R>(L, odd, out, s); break;
    case PLBGPU_BF16: stateOut<__nv_bfloat16, R>(L, odd, out, s); break;
    case PLBGPU_FP16: stateOut<__half, R>(L, odd, out, s); break;
    default: stateOut<bf16sr, R>(L, odd, out, s); break;
    }
}

template <typename R>
void stateInAny(int prec, const DevLattice& L, const R* in, cudaStream_t s) {
    dim3 g = cellGrid(L);
    switch (prec) {
    case PLBGPU_FP64: stateInKernel<double, R><<<g, cellBlock(L), 0, s>>>(L, in); break;
    case PLBGPU_FP32: stateInKernel<float, R><<<g, cellBlock(L), 0, s>>>(L, in); break;
    case PLBGPU_BF16: stateInKernel<__nv_bfloat16, R><<<g, cellBlock(L), 0, s>>>(L, in); break;
    case PLBGPU_FP16: stateInKernel<__half, R><<<g, cellBlock(L), 0, s>>>(L, in); break;
    default: stateInKernel<bf16sr, R><<<g, cellBlock(L), 0, s>>>(L, in); break;
    }
}

// Objective of a sweep: the velocity mismatch (v = u*), a weighted velocity
// (v = w), or the momentum-exchange drag along dir.
enum { kMismatch = 0, kWeighted = 1, kDrag = 2 };
struct Objective {
    int kind = kMismatch;
    const double* v = nullptr;   // host, 3 values per cell (velocity objectives)
    size_t nv = 0;
    double dir[3] = {0., 0., 0.};
};

int checkObjective(plbgpu_ctx* c, const DomainAccess& a, const Objective& o) {
    if (o.kind == kDrag) {
        if (!a.L.mebb)
            return domainFail(c, PLBGPU_ERR_STATE, "adjoint: the drag objective needs initialize_momentum_exchange");
        return PLBGPU_OK;
    }
    if (!o.v || (long long)o.nv != 3 * a.L.n)
        return domainFail(c, PLBGPU_ERR_ARG, "adjoint: the objective needs 3 values per cell");
    return PLBGPU_OK;
}

// J, lambda = dJ/df and the explicit dJ/dF for state f; vDev holds the
// objective's per-cell values on the device (velocity objectives).
template <typename R>
void launchObjective(const DomainAccess& a, const Objective& o, const R* f, const double* vDev, R* lam, R* gF,
                     AdjAcc* acc) {
    if (o.kind == kDrag)
        dragObjectiveKernel<R><<<cellGrid(a.L), cellBlock(a.L), 0, a.stream>>>(a.L, f, o.dir[0], o.dir[1], o.dir[2],
                                                                               lam, acc);
    else
        objectiveKernel<R><<<cellGrid(a.L), cellBlock(a.L), 0, a.stream>>>(a.L, f, vDev, o.kind == kWeighted,
                                                                           (R)(1.0 / a.rho0), lam, gF, acc);
    *a.launches += 1;
}

// The adjoint covers BGK, Guo, incompressible BGK, bounce-back,
// momentum-exchange bounce-back, no-dynamics, the regularized and Zou/He face
// cells and the external velocity edges and corners; `faces` (optional)
// receives the face cells' indices.  An edge or corner that reads a
// Guo-forced cell is refused: its rebuilt populations would depend on that
// cell's force through the finite differences, a path the force gradient does
// not follow.
int checkKinds(plbgpu_ctx* c, const DomainAccess& a, std::vector<long long>* faces = nullptr) {
    std::vector<uint8_t> k((size_t)a.L.n);
    if (cudaMemcpyAsync(k.data(), a.L.flags, k.size(), cudaMemcpyDeviceToHost, a.stream) != cudaSuccess ||
        cudaStreamSynchronize(a.stream) != cudaSuccess)
        return domainFail(c, PLBGPU_ERR_CUDA, "reading cell kinds failed");
    const int nx = a.L.nx, ny = a.L.ny, nz = a.L.nz;
    auto kindAt = [&](int x, int y, int z) {
        x = x < 0 ? x + nx : (x >= nx ? x - nx : x);
        y = y < 0 ? y + ny : (y >= ny ? y - ny : y);
        z = z < 0 ? z + nz : (z >= nz ? z - nz : z);
        return (int)k[((size_t)x * ny + y) * nz + z];
    };
    for (size_t i = 0; i < k.size(); ++i) {
        const int v = k[i];
        if (isFace(v)) {
            if (faces) faces->push_back((long long)i);
            continue;
        }
        if (isSurface(v)) {
            const int p[3] = {(int)(i / ((size_t)ny * nz)), (int)((i / nz) % ny), (int)(i % nz)};
            for (int ax = 0; ax < 3; ++ax)
                for (int s = -1; s <= 1; s += 2) {
                    int q[3] = {p[0], p[1], p[2]};
                    q[ax] += s;
                    if (kindAt(q[0], q[1], q[2]) == K_GUO)
                        return domainFail(c, PLBGPU_ERR_ARG,
                                          "adjoint: an edge or corner cell next to a Guo-forced cell is not supported");
                }
            continue;
        }
        if (v != K_BGK && v != K_GUO && v != K_INCBGK && v != K_BB && v != K_MEBB && v != K_NODYN)
            return domainFail(c, PLBGPU_ERR_ARG,
                              "the adjoint supports BGK, Guo, incompressible BGK, bounce-back, momentum-exchange, "
                              "no-dynamics, face, edge and corner cells");
    }
    return PLBGPU_OK;
}

// The domain's edge and corner list, copied (the adjoint's run outlives later
// changes of the domain's kinds).
int copySurface(plbgpu_ctx* c, int h, const DomainAccess& a, int4** dst, int* nEdges, int* nCorners) {
    const int4* cells = nullptr;
    int ne = 0, nc = 0;
    int rc = domainSurface(c, h, &cells, &ne, &nc);
    if (rc) return rc;
    cudaFree(*dst);
    *dst = nullptr;
    *nEdges = ne;
    *nCorners = nc;
    if (ne + nc == 0) return PLBGPU_OK;
    if (cudaMalloc(dst, sizeof(int4) * (size_t)(ne + nc)) != cudaSuccess ||
        cudaMemcpyAsync(*dst, cells, sizeof(int4) * (size_t)(ne + nc), cudaMemcpyDeviceToDevice, a.stream) !=
            cudaSuccess)
        return domainFail(c, PLBGPU_ERR_NOMEM, "adjoint: copying the edge and corner list failed");
    return PLBGPU_OK;
}

// The edge processors, then the corner processors, on a natural-order state
// just pushed.
template <typename R, typename T>
void launchSurfaceNat(const DomainAccess& a, const int4* surf, int nEdges, int nCorners, T* buf, T omega,
                      cudaStream_t stream = nullptr) {
    const R invRho0 = (R)(1.0 / a.rho0);
    cudaStream_t s = stream ? stream : a.stream;
    if (nEdges)
        surfaceNatKernel<R, T><<<(nEdges + 63) / 64, 64, 0, s>>>(a.L, buf, surf, nEdges, invRho0, a.bbRho, omega);
    if (nCorners)
        surfaceNatKernel<R, T><<<(nCorners + 63) / 64, 64, 0, s>>>(a.L, buf, surf + nEdges, nCorners, invRho0,
                                                                   a.bbRho, omega);
    *a.launches += (nEdges ? 1 : 0) + (nCorners ? 1 : 0);
}

// Their reverse on lambda at the state f they produced: corners first.
template <typename R>
void launchSurfaceAdjoint(const DomainAccess& a, const int4* surf, int nEdges, int nCorners, const R* f, R* lam,
                          AdjAcc* acc) {
    const R invRho0 = (R)(1.0 / a.rho0), omega = (R)a.omega;
    auto reverse = [&](const int4* cells, int count, bool edge) {
        const int passes = surfacePasses(edge);
        const long long threads = (long long)count * passes;
        surfaceAdjointKernel<R><<<(unsigned)((threads + 127) / 128), 128, 0, a.stream>>>(
            a.L, f, lam, cells, count, passes, invRho0, a.bbRho, omega, acc);
        *a.launches += 1;
    };
    if (nCorners) reverse(surf + nEdges, nCorners, false);
    if (nEdges) reverse(surf, nEdges, true);
    if (nEdges + nCorners) {
        surfaceAdjointZero<R><<<(nEdges + nCorners + 127) / 128, 128, 0, a.stream>>>(a.L, lam, surf,
                                                                                     nEdges + nCorners);
        *a.launches += 1;
    }
}

// The face cells' reverse step beside the bulk's (disjoint writes).
template <typename R>
void launchFaceAdjoint(const DomainAccess& a, const long long* faces, int nFaces, const R* f, const R* lamIn,
                       R* lamOut, bool pending, AdjAcc* acc) {
    if (nFaces == 0) return;
    faceAdjointKernel<R><<<(nFaces + 127) / 128, 128, 0, a.stream>>>(a.L, f, lamIn, lamOut, a.omega, pending, faces,
                                                                       nFaces, acc);
    *a.launches += 1;
}

#define ADJ_TRY(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) {                                                               \
            char m_[256];                                                                      \
            snprintf(m_, sizeof(m_), "%s failed: %s", #call, cudaGetErrorString(e_));          \
            return domainFail(c, e_ == cudaErrorMemoryAllocation ? PLBGPU_ERR_NOMEM : PLBGPU_ERR_CUDA, m_); \
        }                                                                                      \
    } while (0)

template <typename R>
int forwardImpl(plbgpu_ctx* c, int h, DomainAccess& a, AdjointState* st, int T, int K) {
    const long long n = a.L.n, sz = 19 * n;
    R* ck = static_cast<R*>(st->ckpt);
    R* sg = static_cast<R*>(st->seg);
    stateOutAny<R>(a.precision, a.L, a.odd, ck, a.stream);
    *a.launches += 1;
    R* cur = ck;
    R* bufs[2] = {sg, sg + sz};
    const R omega = (R)a.omega, invRho0 = (R)(1.0 / a.rho0);
    const NeighbourDeltas D = deltasOf(a.L);
    for (int t = 0; t < T; ++t) {
        R* out = ((t + 1) % K == 0) ? ck + ((t + 1) / K) * sz : bufs[t & 1];
        pushStepKernel<R><<<cellGrid(a.L), cellBlock(a.L), 0, a.stream>>>(a.L, D, cur, out, omega, invRho0, nullptr,
                                                                          st->pendingAt(t));
        *a.launches += 1;
        launchSurfaceNat<R, R>(a, st->surf, st->nEdges, st->nCorners, out, omega);
        cur = out;
    }
    ADJ_TRY(cudaGetLastError());
    // the domain continues from f^T, in natural order
    stateInAny<R>(a.precision, a.L, cur, a.stream);
    *a.launches += 1;
    ADJ_TRY(cudaGetLastError());
    ADJ_TRY(cudaStreamSynchronize(a.stream));
    // the last push streamed: face cells are completed at the next collision
    domainSetState(c, h, false, st->nFaces > 0);
    return PLBGPU_OK;
}

// Capture the launches `enqueue` makes on stream s into an executable graph;
// nullptr when the capture or instantiation fails (nothing was launched then).
template <class F>
cudaGraphExec_t captureGraph(cudaStream_t s, F&& enqueue) {
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    enqueue();
    cudaGraph_t g = nullptr;
    cudaGraphExec_t exec = nullptr;
    if (cudaStreamEndCapture(s, &g) != cudaSuccess || cudaGraphInstantiate(&exec, g, 0) != cudaSuccess)
        exec = nullptr;
    if (g) cudaGraphDestroy(g);
    (void)cudaGetLastError();
    return exec;
}

template <typename R>
int backwardImpl(DomainAccess& a, AdjointState* st, const Objective& o, double* objective, double* gOmega,
                 float* ms) {
    const long long n = a.L.n, sz = 19 * n;
    R* ck = static_cast<R*>(st->ckpt);
    R* sg = static_cast<R*>(st->seg);
    R* lam = static_cast<R*>(st->lam);
    R* gF = static_cast<R*>(st->gF);
    const R omega = (R)a.omega, invRho0 = (R)(1.0 / a.rho0);
    const NeighbourDeltas D = deltasOf(a.L);
    const int T = st->T, K = st->K;
    // Segment s holds f^{sK+1} .. f^{sK+K-1}; with a second segment buffer the
    // side stream recomputes segment s-1 while the main stream reverses
    // segment s (both kernels are latency-bound at a third of the warp slots,
    // so they share the SMs), otherwise each segment is recomputed first.
    R* sg2 = static_cast<R*>(st->seg2);
    const bool overlap = sg2 && st->side && st->fork && st->join && K > 1;
    auto segBuf = [&](int s) { return overlap && (s & 1) ? sg2 : sg; };
    auto stateOf = [&](int s, int k) {
        return k == 0 ? ck + (long long)s * sz : (k == K ? ck + (long long)(s + 1) * sz : segBuf(s) + k * sz);
    };
    auto recompute = [&](int s, cudaStream_t strm) {
        for (int k = 0; k + 1 < K; ++k) {
            pushStepKernel<R><<<cellGrid(a.L), cellBlock(a.L), 0, strm>>>(
                a.L, D, stateOf(s, k), stateOf(s, k + 1), omega, invRho0, nullptr, st->pendingAt((long long)s * K + k));
            *a.launches += 1;
            launchSurfaceNat<R, R>(a, st->surf, st->nEdges, st->nCorners, stateOf(s, k + 1), omega, strm);
        }
    };
    auto sweep = [&]() {
        cudaMemsetAsync(gF, 0, sizeof(R) * 3 * n, a.stream);
        cudaMemsetAsync(st->acc, 0, sizeof(AdjAcc), a.stream);
        launchObjective<R>(a, o, ck + (long long)(T / K) * sz, st->uT, lam, gF, st->acc);
        int cur = 0;   // lam + cur * sz holds lambda^{t+1}
        if (overlap) recompute(T / K - 1, a.stream);
        for (int s = T / K - 1; s >= 0; --s) {
            auto state = [&](int k) { return stateOf(s, k); };
            if (!overlap) {
                recompute(s, a.stream);
            } else if (s > 0) {
                // segment s-1 goes into the buffer segment s+1 used, whose reverse is done
                cudaEventRecord(st->fork, a.stream);
                cudaStreamWaitEvent(st->side, st->fork, 0);
                recompute(s - 1, st->side);
                cudaEventRecord(st->join, st->side);
            }
            for (int k = K - 1; k >= 0; --k) {
                // the edge and corner processors that finished step k, reversed at the state they produced
                launchSurfaceAdjoint<R>(a, st->surf, st->nEdges, st->nCorners, state(k + 1), lam + cur * sz, st->acc);
                adjointStepKernel<R><<<cellGrid(a.L), cellBlock(a.L), 0, a.stream>>>(
                    a.L, D, state(k), lam + cur * sz, lam + (1 - cur) * sz, gF, omega, invRho0, st->acc);
                *a.launches += 1;
                launchFaceAdjoint<R>(a, st->faces, st->nFaces, state(k), lam + cur * sz, lam + (1 - cur) * sz,
                                     st->pendingAt((long long)s * K + k), st->acc);
                cur = 1 - cur;
            }
            if (overlap && s > 0) cudaStreamWaitEvent(a.stream, st->join, 0);   // segment s-1 is ready
        }
    };
    // The sweep is captured once into a CUDA graph and launched as one unit
    // (no host launch gaps between its 2T kernels); without a graph it is
    // launched directly.
    const long long launches0 = *a.launches;
    cudaGraphExec_t exec = captureGraph(a.stream, sweep);
    if (!exec) *a.launches = launches0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, a.stream);
    if (exec) cudaGraphLaunch(exec, a.stream);
    else sweep();
    cudaEventRecord(e1, a.stream);
    cudaEventSynchronize(e1);
    if (ms) cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (exec) cudaGraphExecDestroy(exec);
    AdjAcc h;
    cudaMemcpyAsync(&h, st->acc, sizeof(AdjAcc), cudaMemcpyDeviceToHost, a.stream);
    cudaStreamSynchronize(a.stream);
    *objective = slotSum(h.objective);
    *gOmega = slotSum(h.gOmega);
    return cudaGetLastError() == cudaSuccess ? PLBGPU_OK : PLBGPU_ERR_CUDA;
}

// dJ/dF planes [3][n] on the device -> grad_force [cell][3] in transfer order.
template <typename R>
int forceGradientOut(plbgpu_ctx* c, const DomainAccess& a, const R* gF, double* grad_force) {
    const long long n = a.L.n;
    std::vector<R> planes((size_t)3 * n);
    ADJ_TRY(cudaMemcpyAsync(planes.data(), gF, sizeof(R) * 3 * n, cudaMemcpyDeviceToHost, a.stream));
    ADJ_TRY(cudaStreamSynchronize(a.stream));
    for (long long i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) grad_force[3 * i + d] = (double)planes[d * n + i];
    return PLBGPU_OK;
}

int adjointBackward(plbgpu_ctx* c, int h, const Objective& o, double* objective, double* grad_force, size_t ng,
                    double* grad_omega, float* ms) {
    DomainAccess a;
    int rc = domainAccess(c, h, &a);
    if (rc) return rc;
    AdjointState* st = static_cast<AdjointState*>(*a.adjointSlot);
    if (!st || !st->ready) return domainFail(c, PLBGPU_ERR_STATE, "adjoint: no recorded forward run");
    const long long n = a.L.n;
    if (!objective || !grad_omega) return domainFail(c, PLBGPU_ERR_ARG, "adjoint: objective and grad_omega are NULL");
    if ((rc = checkObjective(c, a, o))) return rc;
    if (grad_force && (long long)ng != 3 * n)
        return domainFail(c, PLBGPU_ERR_ARG, "adjoint: grad_force needs 3 values per cell");
    if (o.kind != kDrag)
        ADJ_TRY(cudaMemcpyAsync(st->uT, o.v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, a.stream));
    rc = a.precision == PLBGPU_FP64 ? backwardImpl<double>(a, st, o, objective, grad_omega, ms)
                                    : backwardImpl<float>(a, st, o, objective, grad_omega, ms);
    if (rc) return domainFail(c, rc, "adjoint: backward sweep failed");
    if (!grad_force) return PLBGPU_OK;
    return a.precision == PLBGPU_FP64 ? forceGradientOut(c, a, static_cast<const double*>(st->gF), grad_force)
                                      : forceGradientOut(c, a, static_cast<const float*>(st->gF), grad_force);
}

// Adjoint of a steady state: the domain's state f is a fixed point of the
// step, so every reverse step linearises around the same f.  The sweep sums
// (d out / d theta)^T lambda over `iterations` reverse steps from
// lambda = dJ/df; the sum converges to the derivative of J at the steady
// state (lambda decays at the rate the flow relaxes; the one mode it keeps,
// total mass, adds nothing because the collision conserves mass for every
// omega and force).  Three states of memory whatever the number of steps.
template <typename R>
int steadyImpl(plbgpu_ctx* c, DomainAccess& a, int iterations, const Objective& o,
               const std::vector<long long>& faceList, const int4* surf, int nEdges, int nCorners, double* objective,
               double* grad_force, double* grad_omega, float* ms) {
    const long long n = a.L.n, sz = 19 * n;
    struct Buffers {
        R* f = nullptr;
        R* lam = nullptr;
        R* gF = nullptr;
        double* w = nullptr;
        AdjAcc* acc = nullptr;
        long long* faces = nullptr;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        ~Buffers() {
            cudaFree(faces);
            cudaFree(f);
            cudaFree(lam);
            cudaFree(gF);
            cudaFree(w);
            cudaFree(acc);
            if (e0) cudaEventDestroy(e0);
            if (e1) cudaEventDestroy(e1);
        }
    } b;
    ADJ_TRY(cudaMalloc(&b.f, sizeof(R) * sz));
    ADJ_TRY(cudaMalloc(&b.lam, sizeof(R) * sz * 2));
    ADJ_TRY(cudaMalloc(&b.gF, sizeof(R) * 3 * n));
    ADJ_TRY(cudaMalloc(&b.w, sizeof(double) * 3 * n));
    ADJ_TRY(cudaMalloc(&b.acc, sizeof(AdjAcc)));
    ADJ_TRY(cudaEventCreate(&b.e0));
    ADJ_TRY(cudaEventCreate(&b.e1));
    const int nFaces = (int)faceList.size();
    if (nFaces) {
        ADJ_TRY(cudaMalloc(&b.faces, sizeof(long long) * faceList.size()));
        ADJ_TRY(cudaMemcpyAsync(b.faces, faceList.data(), sizeof(long long) * faceList.size(), cudaMemcpyHostToDevice,
                                a.stream));
    }
    if (o.kind != kDrag)
        ADJ_TRY(cudaMemcpyAsync(b.w, o.v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, a.stream));
    ADJ_TRY(cudaMemsetAsync(b.gF, 0, sizeof(R) * 3 * n, a.stream));
    ADJ_TRY(cudaMemsetAsync(b.acc, 0, sizeof(AdjAcc), a.stream));
    const R omega = (R)a.omega, invRho0 = (R)(1.0 / a.rho0);
    const NeighbourDeltas D = deltasOf(a.L);
    ADJ_TRY(cudaEventRecord(b.e0, a.stream));
    stateOutAny<R>(a.precision, a.L, a.odd, b.f, a.stream);
    *a.launches += 1;
    launchObjective<R>(a, o, b.f, b.w, b.lam, b.gF, b.acc);
    int cur = 0;
    for (int t = 0; t < iterations; ++t) {
        launchSurfaceAdjoint<R>(a, surf, nEdges, nCorners, b.f, b.lam + cur * sz, b.acc);
        adjointStepKernel<R><<<cellGrid(a.L), cellBlock(a.L), 0, a.stream>>>(a.L, D, b.f, b.lam + cur * sz,
                                                                             b.lam + (1 - cur) * sz, b.gF, omega,
                                                                             invRho0, b.acc);
        *a.launches += 1;
        // the steady state is a streamed state: its faces complete at each step
        launchFaceAdjoint<R>(a, b.faces, nFaces, b.f, b.lam + cur * sz, b.lam + (1 - cur) * sz, nFaces > 0, b.acc);
        cur = 1 - cur;
    }
    ADJ_TRY(cudaGetLastError());
    ADJ_TRY(cudaEventRecord(b.e1, a.stream));
    ADJ_TRY(cudaEventSynchronize(b.e1));
    if (ms) ADJ_TRY(cudaEventElapsedTime(ms, b.e0, b.e1));
    AdjAcc h;
    ADJ_TRY(cudaMemcpyAsync(&h, b.acc, sizeof(AdjAcc), cudaMemcpyDeviceToHost, a.stream));
    ADJ_TRY(cudaStreamSynchronize(a.stream));
    *objective = slotSum(h.objective);
    *grad_omega = slotSum(h.gOmega);
    return grad_force ? forceGradientOut(c, a, b.gF, grad_force) : PLBGPU_OK;
}

int tangentLinear(plbgpu_ctx* c, int h, int T, const double* dforce, size_t ndf, double domega, const Objective& o,
                  double* objective, double* directional) {
    DomainAccess a;
    int rc = domainAccess(c, h, &a);
    if (rc) return rc;
    if (a.precision != PLBGPU_FP64) return domainFail(c, PLBGPU_ERR_ARG, "tangent: FP64 domains only");
    const long long n = a.L.n, sz = 19 * n;
    if (T < 0 || !objective || !directional || (dforce && (long long)ndf != 3 * n))
        return domainFail(c, PLBGPU_ERR_ARG, "tangent: bad arguments");
    if ((rc = checkObjective(c, a, o))) return rc;
    std::vector<long long> faceList;
    if ((rc = checkKinds(c, a, &faceList))) return rc;
    const bool hasFaces = !faceList.empty();
    struct SurfList {
        int4* p = nullptr;
        ~SurfList() { cudaFree(p); }
    } surf;
    int ne = 0, nc = 0;
    if ((rc = copySurface(c, h, a, &surf.p, &ne, &nc))) return rc;
    double *f0 = nullptr, *dF = nullptr, *uT = nullptr;
    Dual* buf = nullptr;
    AdjAcc* acc = nullptr;
    std::vector<double> planes((size_t)3 * n, 0.);
    if (dforce)
        for (long long i = 0; i < n; ++i)
            for (int d = 0; d < 3; ++d) planes[d * n + i] = dforce[3 * i + d];
    cudaError_t e = cudaMalloc(&f0, sizeof(double) * sz);
    if (e == cudaSuccess) e = cudaMalloc(&buf, sizeof(Dual) * sz * 2);
    if (e == cudaSuccess) e = cudaMalloc(&dF, sizeof(double) * 3 * n);
    if (e == cudaSuccess) e = cudaMalloc(&uT, sizeof(double) * 3 * n);
    if (e == cudaSuccess) e = cudaMalloc(&acc, sizeof(AdjAcc));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dF, planes.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice, a.stream);
    if (e == cudaSuccess && o.kind != kDrag)
        e = cudaMemcpyAsync(uT, o.v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, a.stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, sizeof(AdjAcc), a.stream);
    if (e == cudaSuccess) {
        stateOutAny<double>(a.precision, a.L, a.odd, f0, a.stream);
        toDualKernel<double><<<(unsigned)((sz + 255) / 256), 256, 0, a.stream>>>(sz, f0, buf);
        *a.launches += 2;
        Dual* cur = buf;
        Dual* nxt = buf + sz;
        const Dual om(a.omega, domega), inv0(1.0 / a.rho0);
        const NeighbourDeltas D = deltasOf(a.L);
        for (int t = 0; t < T; ++t) {
            pushStepKernel<Dual><<<cellGrid(a.L), cellBlock(a.L), 0, a.stream>>>(a.L, D, cur, nxt, om, inv0, dF,
                                                                                 t == 0 ? a.pending : hasFaces);
            *a.launches += 1;
            launchSurfaceNat<double, Dual>(a, surf.p, ne, nc, nxt, om);
            std::swap(cur, nxt);
        }
        if (o.kind == kDrag)
            dualDragObjectiveKernel<<<cellGrid(a.L), cellBlock(a.L), 0, a.stream>>>(a.L, cur, o.dir[0], o.dir[1],
                                                                                    o.dir[2], acc);
        else
            dualObjectiveKernel<<<cellGrid(a.L), cellBlock(a.L), 0, a.stream>>>(a.L, cur, dF, uT, o.kind == kWeighted,
                                                                                1.0 / a.rho0, acc);
        *a.launches += 1;
        e = cudaGetLastError();
        AdjAcc hacc;
        if (e == cudaSuccess) e = cudaMemcpyAsync(&hacc, acc, sizeof(AdjAcc), cudaMemcpyDeviceToHost, a.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(a.stream);
        if (e == cudaSuccess) {
            *objective = slotSum(hacc.objective);
            *directional = slotSum(hacc.tangent);
        }
    }
    cudaFree(f0); cudaFree(buf); cudaFree(dF); cudaFree(uT); cudaFree(acc);
    if (e != cudaSuccess) {
        char m[256];
        snprintf(m, sizeof(m), "tangent: %s", cudaGetErrorString(e));
        return domainFail(c, e == cudaErrorMemoryAllocation ? PLBGPU_ERR_NOMEM : PLBGPU_ERR_CUDA, m);
    }
    return PLBGPU_OK;
}

}  // namespace
}  // namespace plbgpu

using namespace plbgpu;

extern "C" {

int plbgpu_adjoint_forward(plbgpu_ctx* c, int h, int T, int K) {
    DomainAccess a;
    int rc = domainAccess(c, h, &a);
    if (rc) return rc;
    if (T < 1 || K < 0 || (K > 0 && T % K != 0))
        return domainFail(c, PLBGPU_ERR_ARG, "adjoint: need T >= 1 and K = 0 or a divisor of T");
    std::vector<long long> faces;
    if ((rc = checkKinds(c, a, &faces))) return rc;
    AdjointState* st = static_cast<AdjointState*>(*a.adjointSlot);
    const size_t rs = a.precision == PLBGPU_FP64 ? sizeof(double) : sizeof(float);
    const long long n = a.L.n, sz = 19 * n;
    // states held: T/K + 1 checkpoints, a segment of K recomputed states
    // (none when every step is a checkpoint) and two adjoint states
    auto states = [&](int k) { return (long long)(T / k + 1) + (k > 1 ? std::max(k, 2) : 0) + 2; };
    if (K == 0) {
        // the smallest interval whose states fit in 80% of the free memory
        if (st) {
            freeAdjoint(st);
            *a.adjointSlot = nullptr;
            st = nullptr;
        }
        size_t freeB = 0, totalB = 0;
        ADJ_TRY(cudaMemGetInfo(&freeB, &totalB));
        const double budget = 0.8 * (double)freeB - (double)(rs * 3 + sizeof(double) * 3) * n;
        for (int k = 1; k <= T && K == 0; ++k)
            if (T % k == 0 && (double)states(k) * rs * sz <= budget) K = k;
        if (K == 0) return domainFail(c, PLBGPU_ERR_NOMEM, "adjoint: no checkpoint interval fits in device memory");
    }
    const int nckpt = T / K + 1;
    if (!st || st->precision != a.precision || st->n != n || st->nckpt != nckpt || st->K != K) {
        if (st) freeAdjoint(st);
        *a.adjointSlot = nullptr;
        st = new (std::nothrow) AdjointState();
        if (!st) return domainFail(c, PLBGPU_ERR_NOMEM, "adjoint: host allocation failed");
        *a.adjointSlot = st;
        *a.adjointFree = freeAdjoint;
        st->precision = a.precision;
        st->n = n;
        st->nckpt = nckpt;
        st->K = K;
        ADJ_TRY(cudaMalloc(&st->ckpt, rs * sz * nckpt));
        if (K > 1) {
            ADJ_TRY(cudaMalloc(&st->seg, rs * sz * std::max(K, 2)));
            // a second segment where memory allows: recomputation beside the reverse
            size_t freeB = 0, totalB = 0;
            if (cudaMemGetInfo(&freeB, &totalB) == cudaSuccess &&
                (double)freeB > 1.25 * (double)(rs * sz * (size_t)std::max(K, 2)) &&
                cudaMalloc(&st->seg2, rs * sz * std::max(K, 2)) == cudaSuccess &&
                cudaStreamCreateWithFlags(&st->side, cudaStreamNonBlocking) == cudaSuccess &&
                cudaEventCreateWithFlags(&st->fork, cudaEventDisableTiming) == cudaSuccess &&
                cudaEventCreateWithFlags(&st->join, cudaEventDisableTiming) == cudaSuccess) {
            } else {
                (void)cudaGetLastError();
            }
        }
        ADJ_TRY(cudaMalloc(&st->lam, rs * sz * 2));
        ADJ_TRY(cudaMalloc(&st->gF, rs * 3 * n));
        ADJ_TRY(cudaMalloc(&st->uT, sizeof(double) * 3 * n));
        ADJ_TRY(cudaMalloc(&st->acc, sizeof(AdjAcc)));
    }
    st->T = T;
    st->ready = false;
    if ((rc = copySurface(c, h, a, &st->surf, &st->nEdges, &st->nCorners))) return rc;
    cudaFree(st->faces);
    st->faces = nullptr;
    st->nFaces = (int)faces.size();
    st->pending0 = a.pending;
    if (!faces.empty()) {
        ADJ_TRY(cudaMalloc(&st->faces, sizeof(long long) * faces.size()));
        ADJ_TRY(cudaMemcpyAsync(st->faces, faces.data(), sizeof(long long) * faces.size(), cudaMemcpyHostToDevice,
                                a.stream));
    }
    rc = a.precision == PLBGPU_FP64 ? forwardImpl<double>(c, h, a, st, T, K) : forwardImpl<float>(c, h, a, st, T, K);
    if (rc == PLBGPU_OK) st->ready = true;
    return rc;
}

int plbgpu_adjoint_interval(plbgpu_ctx* c, int h, int* K) {
    DomainAccess a;
    int rc = domainAccess(c, h, &a);
    if (rc) return rc;
    const AdjointState* st = static_cast<const AdjointState*>(*a.adjointSlot);
    if (!K) return domainFail(c, PLBGPU_ERR_ARG, "adjoint: K is NULL");
    if (!st || !st->ready) return domainFail(c, PLBGPU_ERR_STATE, "adjoint: no recorded forward run");
    *K = st->K;
    return PLBGPU_OK;
}

int plbgpu_adjoint_backward(plbgpu_ctx* c, int h, const double* u_target, size_t n3, double* objective,
                            double* grad_force, size_t ng, double* grad_omega, float* ms) {
    Objective o;
    o.v = u_target;
    o.nv = n3;
    return adjointBackward(c, h, o, objective, grad_force, ng, grad_omega, ms);
}

int plbgpu_adjoint_backward_weighted(plbgpu_ctx* c, int h, const double* weights, size_t n3, double* objective,
                                     double* grad_force, size_t ng, double* grad_omega, float* ms) {
    Objective o;
    o.kind = kWeighted;
    o.v = weights;
    o.nv = n3;
    return adjointBackward(c, h, o, objective, grad_force, ng, grad_omega, ms);
}

int plbgpu_adjoint_backward_drag(plbgpu_ctx* c, int h, const double* direction, double* objective, double* grad_force,
                                 size_t ng, double* grad_omega, float* ms) {
    if (!direction) return domainFail(c, PLBGPU_ERR_ARG, "adjoint: direction is NULL");
    Objective o;
    o.kind = kDrag;
    for (int d = 0; d < 3; ++d) o.dir[d] = direction[d];
    return adjointBackward(c, h, o, objective, grad_force, ng, grad_omega, ms);
}

static int adjointSteady(plbgpu_ctx* c, int h, int iterations, const Objective& o, double* objective,
                         double* grad_force, size_t ng, double* grad_omega, float* ms) {
    DomainAccess a;
    int rc = domainAccess(c, h, &a);
    if (rc) return rc;
    const long long n = a.L.n;
    if (iterations < 0 || !objective || !grad_omega || (grad_force && (long long)ng != 3 * n))
        return domainFail(c, PLBGPU_ERR_ARG, "steady adjoint: bad arguments");
    if ((rc = checkObjective(c, a, o))) return rc;
    std::vector<long long> faces;
    if ((rc = checkKinds(c, a, &faces))) return rc;
    int4* surf = nullptr;
    int ne = 0, nc = 0;
    if ((rc = copySurface(c, h, a, &surf, &ne, &nc))) return rc;
    rc = a.precision == PLBGPU_FP64
             ? steadyImpl<double>(c, a, iterations, o, faces, surf, ne, nc, objective, grad_force, grad_omega, ms)
             : steadyImpl<float>(c, a, iterations, o, faces, surf, ne, nc, objective, grad_force, grad_omega, ms);
    cudaStreamSynchronize(a.stream);
    cudaFree(surf);
    return rc;
}

int plbgpu_adjoint_steady_weighted(plbgpu_ctx* c, int h, int iterations, const double* weights, size_t n3,
                                   double* objective, double* grad_force, size_t ng, double* grad_omega, float* ms) {
    Objective o;
    o.kind = kWeighted;
    o.v = weights;
    o.nv = n3;
    return adjointSteady(c, h, iterations, o, objective, grad_force, ng, grad_omega, ms);
}

int plbgpu_adjoint_steady_drag(plbgpu_ctx* c, int h, int iterations, const double* direction, double* objective,
                               double* grad_force, size_t ng, double* grad_omega, float* ms) {
    if (!direction) return domainFail(c, PLBGPU_ERR_ARG, "steady adjoint: direction is NULL");
    Objective o;
    o.kind = kDrag;
    for (int d = 0; d < 3; ++d) o.dir[d] = direction[d];
    return adjointSteady(c, h, iterations, o, objective, grad_force, ng, grad_omega, ms);
}

int plbgpu_tangent_linear(plbgpu_ctx* c, int h, int T, const double* dforce, size_t ndf, double domega,
                          const double* u_target, size_t n3, double* objective, double* directional) {
    Objective o;
    o.v = u_target;
    o.nv = n3;
    return tangentLinear(c, h, T, dforce, ndf, domega, o, objective, directional);
}

int plbgpu_tangent_linear_weighted(plbgpu_ctx* c, int h, int T, const double* dforce, size_t ndf, double domega,
                                   const double* weights, size_t n3, double* objective, double* directional) {
    Objective o;
    o.kind = kWeighted;
    o.v = weights;
    o.nv = n3;
    return tangentLinear(c, h, T, dforce, ndf, domega, o, objective, directional);
}

int plbgpu_tangent_linear_drag(plbgpu_ctx* c, int h, int T, const double* dforce, size_t ndf, double domega,
                               const double* direction, double* objective, double* directional) {
    if (!direction) return domainFail(c, PLBGPU_ERR_ARG, "tangent: direction is NULL");
    Objective o;
    o.kind = kDrag;
    for (int d = 0; d < 3; ++d) o.dir[d] = direction[d];
    return tangentLinear(c, h, T, dforce, ndf, domega, o, objective, directional);
}

}  // extern "C"
