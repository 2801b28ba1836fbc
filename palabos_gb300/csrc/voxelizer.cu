// Mesh voxelizer: voxel flags of a closed triangle mesh on an nx*ny*nz box,
// the result of the reference's voxelize(mesh, domain, borderWidth)
// (offLattice/voxelizer.hh:106-141) with DetectBorderLineFunctional3D
// (voxelizer.hh:653-685).  Flags: 1 outside, 2 outerBorder, 3 inside,
// 4 innerBorder.
//
// The reference seeds the box's outer layer "outside" and floods inwards: a
// cell takes a determined neighbour's flag, inverted when the segment between
// the two crosses the surface an odd number of times.  On the GPU every
// (y, z) column with 1 <= y <= ny-2, 1 <= z <= nz-2 is one thread that walks
// the same flood along x from its seeded cell x = 0: it gathers the
// crossings of its line with the triangles binned to the column, and flips
// the flag at each unit segment (x-1, x] holding an odd number of them.  For
// a closed surface every path of the flood gives the same parity, so this is
// the reference's result.  Ties follow the reference's conventions:
//   * a line through a shared edge or vertex is counted once: the
//     point-in-triangle test in the (y, z) plane evaluates each edge in one
//     canonical direction and breaks exact zeros by a fixed symbolic shift of
//     the point, so exactly one of the triangles around an edge or vertex
//     claims it (the reference merges crossings at equal distances);
//   * a cell centre on the surface lies behind it: the reference shifts the
//     triangle by 2 eps1 along its normal, so the crossing goes to the
//     segment after the cell when the normal's x component is positive.
// Borders: an outside cell with an inside cell within borderWidth (box
// neighbourhood, inside the lattice) becomes outerBorder, an inside cell with
// an outside one innerBorder.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <vector>

#include <cuda_runtime.h>

#include "launch.h"
#include "plbgpu.h"

namespace plbgpu {
namespace {

constexpr int kMaxCrossings = 64;   // per column; more is reported as an error
constexpr int kMaxRuns = 32;        // disjoint runs of on-surface cells per column; more is an error
constexpr int kVxOutside = 1, kVxOuterBorder = 2, kVxInside = 3, kVxInnerBorder = 4;
constexpr unsigned kTooManyCrossings = 1u, kTooManyRuns = 2u;   // status bits

// The cells x = lo..hi of a column lie on the surface (hence inside).  Runs
// are kept disjoint and merged as they arrive -- overlapping or touching runs
// become one -- so a finely meshed face that many facets cover counts once.
// Returns false when a new disjoint run does not fit.
__device__ bool addRun(int* runLo, int* runHi, int& m, int lo, int hi) {
    for (int k = 0; k < m;) {
        if (lo <= runHi[k] + 1 && runLo[k] <= hi + 1) {   // overlap or touch: absorb run k
            lo = min(lo, runLo[k]);
            hi = max(hi, runHi[k]);
            --m;
            runLo[k] = runLo[m];
            runHi[k] = runHi[m];
        } else {
            ++k;
        }
    }
    if (m == kMaxRuns) return false;
    runLo[m] = lo;
    runHi[m] = hi;
    ++m;
    return true;
}

// Sign of the orientation of p against the edge u -> v in the (y, z) plane,
// never zero: the edge is evaluated from its lexicographically smaller end
// and an exact zero takes the sign p would have after a shift by
// (epsilon, epsilon^2).
__device__ __forceinline__ int edgeSide(double uy, double uz, double vy, double vz, double py, double pz) {
    const bool swap = vy < uy || (vy == uy && vz < uz);
    if (swap) {
        double t = uy; uy = vy; vy = t;
        t = uz; uz = vz; vz = t;
    }
    const double dy = vy - uy, dz = vz - uz;
    const double e = dy * (pz - uz) - dz * (py - uy);
    int s = e > 0. ? 1 : (e < 0. ? -1 : 0);
    if (s == 0) s = dz != 0. ? (dz > 0. ? -1 : 1) : (dy > 0. ? 1 : -1);
    return swap ? -s : s;
}

// The x-range where the line {(x, py, pz)} meets triangle T, whose (y, z)
// projection is a segment or a point (a facet parallel to x); false when the
// line misses it.
__device__ bool facetSpan(const double* T, double py, double pz, double scale, double& lo, double& hi) {
    const double tol = 1e-12 * scale;
    bool any = false;
    lo = 1e300;
    hi = -1e300;
    for (int e = 0; e < 3; ++e) {
        const double* U = T + 3 * e;
        const double* V = T + 3 * ((e + 1) % 3);
        const double dy = V[1] - U[1], dz = V[2] - U[2];
        const double len2 = dy * dy + dz * dz;
        double xs[2];
        int nxs = 0;
        if (len2 <= tol * tol) {   // the edge runs along x
            if (fabs(py - U[1]) <= tol && fabs(pz - U[2]) <= tol) {
                xs[0] = U[0];
                xs[1] = V[0];
                nxs = 2;
            }
        } else {
            const double cross = dy * (pz - U[2]) - dz * (py - U[1]);
            const double t = (dy * (py - U[1]) + dz * (pz - U[2])) / len2;
            if (fabs(cross) <= tol * sqrt(len2) && t >= -1e-12 && t <= 1. + 1e-12) {
                xs[0] = U[0] + t * (V[0] - U[0]);
                nxs = 1;
            }
        }
        for (int i = 0; i < nxs; ++i) {
            lo = fmin(lo, xs[i]);
            hi = fmax(hi, xs[i]);
            any = true;
        }
    }
    return any;
}

__global__ void columnKernel(int nx, int ny, int nz, const double* tri, const int* start, const int* list,
                             int32_t* flags, unsigned* status) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (z >= nz) return;
    const long long plane = (long long)ny * nz;
    const long long col = (long long)y * nz + z;
    if (y == 0 || y == ny - 1 || z == 0 || z == nz - 1) {
        for (int x = 0; x < nx; ++x) flags[x * plane + col] = kVxOutside;
        return;
    }
    const double py = y, pz = z;
    int seg[kMaxCrossings];   // the crossing lies in the unit segment (seg - 1, seg]
    int m = 0;
    int runLo[kMaxRuns], runHi[kMaxRuns];   // disjoint runs of cells on the surface
    int m2 = 0;
    // cells x (1 <= x <= nx-2, the flooded interior) with lo - 1e-12 <= x <= hi + 1e-12
    auto onSurface = [&](double lo, double hi) {
        const double a = fmax(1., ceil(lo - 1e-12)), b = fmin((double)(nx - 2), floor(hi + 1e-12));
        if (a <= b && !addRun(runLo, runHi, m2, (int)a, (int)b)) atomicOr(status, kTooManyRuns);
    };
    const int c = y * nz + z;
    for (int k = start[c]; k < start[c + 1]; ++k) {
        const double* T = tri + 9 * (long long)list[k];
        const double ax = T[0], ay = T[1], az = T[2], bx = T[3], by = T[4], bz = T[5], cx = T[6], cy = T[7],
                     cz = T[8];
        const double area = (by - ay) * (cz - az) - (bz - az) * (cy - ay);   // x component of the normal
        const double scale = fmax(1., fmax(fabs(ay) + fabs(by) + fabs(cy), fabs(az) + fabs(bz) + fabs(cz)));
        const double tol = 1e-12 * scale * scale;
        if (fabs(area) <= tol) {
            // a facet parallel to x: the cells of the line that lie on it are
            // on the surface, hence inside
            double lo, hi;
            if (facetSpan(T, py, pz, scale, lo, hi)) onSurface(lo, hi);
            continue;
        }
        const double wa = (cy - by) * (pz - bz) - (cz - bz) * (py - by);
        const double wb = (ay - cy) * (pz - cz) - (az - cz) * (py - cy);
        const double wc = (by - ay) * (pz - az) - (bz - az) * (py - ay);
        const double xi = (wa * ax + wb * bx + wc * cx) / (wa + wb + wc);
        const double r = nearbyint(xi);
        const bool centre = fabs(xi - r) <= 1e-12 * fmax(1., fabs(xi));
        // a cell centre on the closed facet (edges and vertices too, where the
        // line may only touch the surface) is on the surface, hence inside
        const bool closed = area > 0. ? (wa >= -tol && wb >= -tol && wc >= -tol) : (wa <= tol && wb <= tol && wc <= tol);
        if (closed && centre && r >= 0. && r <= (double)nx) onSurface(r, r);
        const int s1 = edgeSide(ay, az, by, bz, py, pz);
        const int s2 = edgeSide(by, bz, cy, cz, py, pz);
        const int s3 = edgeSide(cy, cz, ay, az, py, pz);
        if (s1 != s2 || s2 != s3) continue;
        if (!(xi > -1.) || xi > (double)nx + 1.) continue;   // beyond the box along x
        int s;
        if (centre) s = (int)r + (area > 0. ? 1 : 0);   // on a cell centre
        else s = (int)ceil(xi);
        if (s < 1 || s > nx - 2) continue;   // segments outside the flooded interior
        if (m == kMaxCrossings) {
            atomicOr(status, kTooManyCrossings);
            break;
        }
        seg[m++] = s;
    }
    // insertion sort of the few crossings, then the flood along x
    for (int i = 1; i < m; ++i) {
        const int v = seg[i];
        int j = i - 1;
        while (j >= 0 && seg[j] > v) {
            seg[j + 1] = seg[j];
            --j;
        }
        seg[j + 1] = v;
    }
    bool inside = false;
    int next = 0;
    flags[col] = kVxOutside;
    for (int x = 1; x < nx - 1; ++x) {
        while (next < m && seg[next] == x) {
            inside = !inside;
            ++next;
        }
        bool on = false;
        for (int k = 0; k < m2; ++k) on |= x >= runLo[k] && x <= runHi[k];
        flags[x * plane + col] = (inside || on) ? kVxInside : kVxOutside;
    }
    if (nx > 1) flags[(nx - 1) * plane + col] = kVxOutside;
}

__device__ __forceinline__ bool vxInside(int f) { return f == kVxInside || f == kVxInnerBorder; }

__global__ void borderKernel(int nx, int ny, int nz, int bw, const int32_t* bulk, int32_t* flags) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    if (z >= nz) return;
    const long long id = ((long long)x * ny + y) * nz + z;
    const bool in = vxInside(bulk[id]);
    bool other = false;
    for (int dx = -bw; dx <= bw && !other; ++dx)
        for (int dy = -bw; dy <= bw && !other; ++dy)
            for (int dz = -bw; dz <= bw && !other; ++dz) {
                const int X = x + dx, Y = y + dy, Z = z + dz;
                if ((dx | dy | dz) == 0 || X < 0 || Y < 0 || Z < 0 || X >= nx || Y >= ny || Z >= nz) continue;
                other = vxInside(bulk[((long long)X * ny + Y) * nz + Z]) != in;
            }
    flags[id] = in ? (other ? kVxInnerBorder : kVxInside) : (other ? kVxOuterBorder : kVxOutside);
}

}  // namespace
}  // namespace plbgpu

using namespace plbgpu;

extern "C" int plbgpu_voxelize(plbgpu_ctx* c, const double* triangles, size_t n_triangles, int nx, int ny, int nz,
                               int border_width, int32_t* flags, size_t n) {
    if (!c) return PLBGPU_ERR_ARG;
    if (nx < 1 || ny < 1 || nz < 1 || nx > 65535 || ny > 65535 || border_width < 0 || !flags ||
        n != (size_t)nx * ny * nz || (n_triangles && !triangles) || n_triangles > (size_t)INT32_MAX ||
        (long long)ny * nz > INT32_MAX)
        return domainFail(c, PLBGPU_ERR_ARG, "voxelize: bad arguments");
    for (size_t i = 0; i < 9 * n_triangles; ++i)
        if (!std::isfinite(triangles[i])) return domainFail(c, PLBGPU_ERR_ARG, "voxelize: a vertex is not finite");
    // bin the triangles to the (y, z) lattice columns their projection covers
    // (counted in 64 bits; the device lists take at most INT32_MAX entries)
    const int ncol = ny * nz;
    std::vector<long long> count((size_t)ncol + 1, 0);
    std::vector<int> start, list;
    auto span = [&](int t, int a, int dim, int& lo, int& hi) {
        const double* T = triangles + 9 * (size_t)t;
        const double mn = std::min(T[a], std::min(T[3 + a], T[6 + a])), mx = std::max(T[a], std::max(T[3 + a], T[6 + a]));
        lo = (int)std::max(0., std::min((double)dim, std::ceil(mn - 1e-9)));
        hi = (int)std::min((double)dim - 1., std::max(-1., std::floor(mx + 1e-9)));
    };
    for (int pass = 0; pass < 2; ++pass) {
        std::vector<long long> fill;
        if (pass == 1) {
            for (int k = 0; k < ncol; ++k) count[k + 1] += count[k];
            if (count[ncol] > (long long)INT32_MAX)
                return domainFail(c, PLBGPU_ERR_ARG,
                                  "voxelize: the triangles cover more than 2^31-1 (triangle, lattice line) pairs");
            start.assign(count.begin(), count.end());
            list.resize((size_t)count[ncol]);
            fill.assign(count.begin(), count.end() - 1);
        }
        for (int t = 0; t < (int)n_triangles; ++t) {
            int y0, y1, z0, z1;
            span(t, 1, ny, y0, y1);
            span(t, 2, nz, z0, z1);
            for (int y = y0; y <= y1; ++y)
                for (int z = z0; z <= z1; ++z) {
                    if (pass == 0) ++count[(size_t)y * nz + z + 1];
                    else list[(size_t)fill[(size_t)y * nz + z]++] = t;
                }
        }
    }
    cudaStream_t s = contextStream(c);
    double* dTri = nullptr;
    int *dStart = nullptr, *dList = nullptr;
    int32_t *dBulk = nullptr, *dFlags = nullptr;
    unsigned* dStatus = nullptr;
    cudaError_t e = cudaMalloc(&dTri, sizeof(double) * 9 * std::max<size_t>(n_triangles, 1));
    if (e == cudaSuccess) e = cudaMalloc(&dStart, sizeof(int) * start.size());
    if (e == cudaSuccess) e = cudaMalloc(&dList, sizeof(int) * std::max<size_t>(list.size(), 1));
    if (e == cudaSuccess) e = cudaMalloc(&dBulk, sizeof(int32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&dFlags, sizeof(int32_t) * n);
    if (e == cudaSuccess) e = cudaMalloc(&dStatus, sizeof(unsigned));
    if (e == cudaSuccess && n_triangles)
        e = cudaMemcpyAsync(dTri, triangles, sizeof(double) * 9 * n_triangles, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dStart, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !list.empty())
        e = cudaMemcpyAsync(dList, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dStatus, 0, sizeof(unsigned), s);
    unsigned status = 0;
    if (e == cudaSuccess) {
        const int tpb = 128;
        columnKernel<<<dim3((unsigned)((nz + tpb - 1) / tpb), (unsigned)ny), tpb, 0, s>>>(nx, ny, nz, dTri, dStart,
                                                                                          dList, dBulk, dStatus);
        borderKernel<<<dim3((unsigned)((nz + tpb - 1) / tpb), (unsigned)ny, (unsigned)nx), tpb, 0, s>>>(
            nx, ny, nz, border_width, dBulk, dFlags);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(flags, dFlags, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, dStatus, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(dTri);
    cudaFree(dStart);
    cudaFree(dList);
    cudaFree(dBulk);
    cudaFree(dFlags);
    cudaFree(dStatus);
    if (e != cudaSuccess) {
        char m[256];
        snprintf(m, sizeof(m), "voxelize: %s", cudaGetErrorString(e));
        return domainFail(c, e == cudaErrorMemoryAllocation ? PLBGPU_ERR_NOMEM : PLBGPU_ERR_CUDA, m);
    }
    if (status & kTooManyCrossings)
        return domainFail(c, PLBGPU_ERR_ARG, "voxelize: a lattice line crosses the surface more than 64 times");
    if (status & kTooManyRuns)
        return domainFail(c, PLBGPU_ERR_ARG,
                          "voxelize: a lattice line lies on the surface in more than 32 separate runs of cells");
    return PLBGPU_OK;
}
