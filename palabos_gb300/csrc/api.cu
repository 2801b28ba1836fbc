// C-ABI implementation (include/plbgpu.h): contexts, domains, transfers,
// time stepping and reductions on one GPU.
//
// A domain is one rectangular lattice in a single device allocation:
//   [ 19 population planes | cell kinds ]
// plus, allocated on first need, the boundary values (3 FP64 planes), the Guo
// force (3 planes, FP64 for the FP64 form and FP32 otherwise), the
// momentum-exchange fluid-direction masks and the list of edge and corner
// cells.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/plbgpu.h"
#include "dynstate.h"
#include "launch.h"

using namespace plbgpu;

namespace {

// NVTX ranges named like the reference profiler's timers
// (core/plbProfiler.h:44-56): "cycle" around a collide-and-stream call
// (MultiBlockLattice3D::collideAndStream, multiBlock/multiBlockLattice3D.hh:319),
// "collStream" around the launches of one time step, with the number of cells
// as payload (the "collStreamCells" counter, atomicBlock/blockLattice3D.hh:
// 257-258), "dataProcessor" around the edge and corner processors
// (multiBlock/multiBlock3D.cpp:487), "io" around transfers and checkpoints.
// The ranges mark host-side submission; without an attached tool they cost
// one branch each.
struct ProfRange {
    explicit ProfRange(const char* name, unsigned long long payload = 0) {
        nvtxEventAttributes_t a = {};
        a.version = NVTX_VERSION;
        a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
        a.messageType = NVTX_MESSAGE_TYPE_ASCII;
        a.message.ascii = name;
        a.payloadType = NVTX_PAYLOAD_TYPE_UNSIGNED_INT64;
        a.payload.ullValue = payload;
        nvtxRangePushEx(&a);
    }
    ~ProfRange() { nvtxRangePop(); }
    ProfRange(const ProfRange&) = delete;
    ProfRange& operator=(const ProfRange&) = delete;
};

// One entry of the data-processor list a lattice state's description carries
// (io/multiBlockWriter3D.cpp:113-136): the processor's registered name, its
// domain, its serialized data, its level and the ids of the blocks it acts
// on.  In the name, "%TD" stands for "double_<Descriptor>" of the saved
// lattice (the reference names its generators after their template
// arguments, e.g. OuterVelocityEdge_double_D3Q19_0_-1_1).
struct ProcessorRecord {
    std::string name, data;
    long long domain[6] = {0, 0, 0, 0, 0, 0};
    long long level = 0;
    std::vector<long long> blocks;
};

struct Domain {
    int nx = 0, ny = 0, nz = 0;
    int precision = PLBGPU_FP64;
    int per[3] = {0, 0, 0};
    double omega = 1.0, rho0 = 1.0, bbRho = 0.0;
    long long n = 0, stride = 0;
    size_t elemSize = 8;
    void* arena = nullptr;       // populations + kinds
    uint8_t* flags = nullptr;
    double* bc = nullptr;        // 3 * n
    void* force = nullptr;       // 3 * n of FP64 or FP32
    void* ext = nullptr;         // 4 * n of FP64 or FP32: external rho-bar, jx, jy, jz
    uint32_t* mebb = nullptr;    // n
    int4* surf = nullptr;        // edge cells, then corner cells: (x, y, z, kind)
    int4* tileLists = nullptr;   // sparse domains: dense, masked, then general tiles (x, y, z0, z1)
    int nDense = 0, nMasked = 0, nGeneral = 0, tileListCap = 0;
    uint32_t* tileMasks = nullptr;   // per cell of the masked tiles: neighbours outside the lattice
    int tileMaskCap = 0;
    int4* rowFaces = nullptr;    // face cells of interior rows (x, y, z, kind), completed before a step
    int nRowFaces = 0, rowFaceCap = 0;
    bool rowFacesDirty = true;   // the list needs rebuilding (kinds changed)
    int surfCap = 0, nEdges = 0, nCorners = 0;
    bool hasSurface = false;     // any edge or corner kind
    bool sparse = false;         // any cell outside the lattice (K_NONE)
    bool surfDirty = false;      // the list needs rebuilding (kinds or periodicity changed)
    StatsAcc* stats = nullptr;   // device accumulators (kStatsSlots of them)
    unsigned* status = nullptr;  // device error word written by the kernels
    ReduceAcc* red = nullptr;
    bool odd = false;            // AA parity of the stored state
    bool pending = false;        // faces still need their post-stream completion
    bool statsValid = false;
    unsigned long long steps = 0;   // time steps taken (salt of stochastic rounding)
    double lastStats[7] = {0, 0, 0, 0, 0, 0, 0};
    unsigned long long deviceBytes = 0;
    void* adjoint = nullptr;              // adjoint checkpoints and buffers (adjoint.cu)
    void (*adjointFree)(void*) = nullptr;
    std::vector<ProcessorRecord> processors;   // the lattice's data-processor list, in order

    DevLattice view() const {
        DevLattice L;
        L.pop = arena;
        L.stride = stride;
        L.flags = flags;
        L.mebb = mebb;
        L.bc = bc;
        L.force = force;
        L.ext = ext;
        L.sparse = sparse ? 1 : 0;
        L.nx = nx; L.ny = ny; L.nz = nz;
        L.per[0] = per[0]; L.per[1] = per[1]; L.per[2] = per[2];
        L.n = n;
        L.status = status;
        L.rowForm = 0;
        L.xRow0 = 0;
        L.xRows = nx - 2;
        L.rowFacesDone = 0;
        const bool lists = sparse && tileLists;
        L.denseTiles = lists && nDense ? tileLists : nullptr;
        L.nDense = lists ? nDense : 0;
        L.maskedTiles = lists && nMasked ? tileLists + nDense : nullptr;
        L.nMasked = lists ? nMasked : 0;
        L.tileMasks = lists && nMasked ? tileMasks : nullptr;
        L.generalTiles = lists && nGeneral ? tileLists + nDense + nMasked : nullptr;
        L.nGeneral = lists ? nGeneral : 0;
        return L;
    }
};

}  // namespace

struct plbgpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    SideStream side = {nullptr, nullptr, nullptr};   // border rows of a step run here
    std::string lastError;
    std::map<int, std::unique_ptr<Domain>> domains;
    int nextHandle = 0;
    unsigned long long launches = 0;
    void* staging = nullptr;     // device staging buffer for transfers
    size_t stagingBytes = 0;
    bool pageableAccess = false; // kernels may dereference pageable host memory (host page tables)
    bool forceStaged = false;    // PLBGPU_STAGED_TRANSFERS=1: always go through the staging buffer
    int rowForm = 0;             // PLBGPU_ROW_KERNEL=cell: one-cell interior-row kernels (DevLattice::rowForm)
    std::vector<cudaEvent_t> slabEvents;   // plbgpu_run_host: four per slab, created on first use
    cudaStream_t xfer = nullptr;           // plbgpu_run_host: the host copies (highest priority, created on first use)
};

namespace {

int fail(plbgpu_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->lastError = buf;
    return code;
}

#define CUDA_TRY(ctx, call)                                                                       \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? PLBGPU_ERR_NOMEM : PLBGPU_ERR_CUDA,  \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                           \
    } while (0)

const Launchers& launchers(int precision) {
    switch (precision) {
    case PLBGPU_FP32: return launchersFp32();
    case PLBGPU_BF16: return launchersBf16();
    case PLBGPU_FP16: return launchersFp16();
    case PLBGPU_BF16_SR: return launchersBf16Sr();
    default: return launchersFp64();
    }
}

size_t elemSizeOf(int precision) {
    return precision == PLBGPU_FP64 ? 8 : precision == PLBGPU_FP32 ? 4 : 2;   // BF16, FP16, BF16_SR: 2
}

int lookup(plbgpu_ctx* c, int h, Domain** d) {
    if (!c) return PLBGPU_ERR_ARG;
    auto it = c->domains.find(h);
    if (it == c->domains.end()) return fail(c, PLBGPU_ERR_HANDLE, "unknown domain handle %d", h);
    *d = it->second.get();
    return PLBGPU_OK;
}

int checkBox(plbgpu_ctx* c, const Domain* d, int x0, int x1, int y0, int y1, int z0, int z1, Box* b) {
    if (x0 < 0 || y0 < 0 || z0 < 0 || x1 >= d->nx || y1 >= d->ny || z1 >= d->nz || x0 > x1 || y0 > y1 ||
        z0 > z1)
        return fail(c, PLBGPU_ERR_ARG, "box [%d,%d]x[%d,%d]x[%d,%d] outside the %dx%dx%d domain", x0, x1, y0,
                    y1, z0, z1, d->nx, d->ny, d->nz);
    b->x0 = x0; b->x1 = x1; b->y0 = y0; b->y1 = y1; b->z0 = z0; b->z1 = z1;
    return PLBGPU_OK;
}

long long boxCells(const Box& b) {
    return (long long)(b.x1 - b.x0 + 1) * (b.y1 - b.y0 + 1) * (b.z1 - b.z0 + 1);
}

int ensureStaging(plbgpu_ctx* c, size_t bytes) {
    if (c->stagingBytes >= bytes) return PLBGPU_OK;
    if (c->staging) {
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        cudaFree(c->staging);
        c->staging = nullptr;
        c->stagingBytes = 0;
    }
    CUDA_TRY(c, cudaMalloc(&c->staging, bytes));
    c->stagingBytes = bytes;
    return PLBGPU_OK;
}

// How the transfer kernels reach a caller's buffer of populations: directly
// when the GPU can address it -- device or managed memory, pinned host memory,
// or, on a GPU that walks the host's page tables (a GB300 next to its Grace
// CPU over NVLink-C2C), plain pageable host memory -- otherwise (nullptr)
// through the bounded staging buffer, chunk by chunk.
const void* directPointer(plbgpu_ctx* c, const void* p) {
    if (c->forceStaged) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    switch (a.type) {
    case cudaMemoryTypeDevice: return a.device == c->device ? a.devicePointer : nullptr;
    case cudaMemoryTypeManaged:
    case cudaMemoryTypeHost: return a.devicePointer;
    default: return c->pageableAccess ? p : nullptr;
    }
}

// Staged transfers move at most this many bytes per copy.
constexpr size_t kStageChunk = size_t(64) << 20;

// The sub-boxes of b (whole x-planes, or rows of one plane when a plane is
// larger than a chunk) whose transfer records fit in one staging chunk, with
// their offset (in doubles) in the box's buffer.  Returns the staging bytes.
template <class Fn>
int forEachChunk(const Box& b, Fn fn, size_t* stageBytes) {
    const long long bny = b.y1 - b.y0 + 1, bnz = b.z1 - b.z0 + 1;
    const size_t rowB = (size_t)bnz * 19 * sizeof(double), planeB = rowB * (size_t)bny;
    if (planeB <= kStageChunk) {
        const int xs = (int)(kStageChunk / planeB);
        *stageBytes = planeB * (size_t)std::min<long long>(xs, b.x1 - b.x0 + 1);
        for (int x = b.x0; x <= b.x1; x += xs) {
            Box s = b;
            s.x0 = x;
            s.x1 = std::min(x + xs - 1, b.x1);
            int rc = fn(s, (size_t)(x - b.x0) * bny * bnz * 19);
            if (rc) return rc;
        }
    } else {
        const int ys = (int)std::max<size_t>(1, kStageChunk / rowB);
        *stageBytes = rowB * (size_t)std::min<long long>(ys, bny);
        for (int x = b.x0; x <= b.x1; ++x)
            for (int y = b.y0; y <= b.y1; y += ys) {
                Box s = b;
                s.x0 = s.x1 = x;
                s.y0 = y;
                s.y1 = std::min(y + ys - 1, b.y1);
                int rc = fn(s, ((size_t)(x - b.x0) * bny + (y - b.y0)) * bnz * 19);
                if (rc) return rc;
            }
    }
    return PLBGPU_OK;
}

// ---------------------------------------------------------------- small kernels

__global__ void fillKindsKernel(uint8_t* flags, int ny, int nz, Box b, uint8_t k) {
    const int bnz = b.z1 - b.z0 + 1;
    const int dz = blockIdx.x * blockDim.x + threadIdx.x;
    if (dz >= bnz) return;
    long long idx = ((long long)(b.x0 + blockIdx.z) * ny + (b.y0 + blockIdx.y)) * nz + b.z0 + dz;
    flags[idx] = k;
}

// Scatter (dir=0) or gather (dir=1) of `comps` values of type V per cell
// between a packed box buffer and `planes` (component c at planes[c*n + idx]).
template <typename V, typename W>
__global__ void boxPlanesKernel(V* planes, long long n, int ny, int nz, Box b, W* packed, int comps,
                                int gather) {
    const int bnz = b.z1 - b.z0 + 1, bny = b.y1 - b.y0 + 1;
    const int dz = blockIdx.x * blockDim.x + threadIdx.x;
    if (dz >= bnz) return;
    long long idx = ((long long)(b.x0 + blockIdx.z) * ny + (b.y0 + blockIdx.y)) * nz + b.z0 + dz;
    long long o = (((long long)blockIdx.z * bny + blockIdx.y) * bnz + dz) * comps;
    for (int c = 0; c < comps; ++c) {
        if (gather) packed[o + c] = (W)planes[c * n + idx];
        else planes[c * n + idx] = (V)packed[o + c];
    }
}

template <typename V>
__global__ void boxPlanesConstKernel(V* planes, long long n, int ny, int nz, Box b, double v0, double v1,
                                     double v2, int comps) {
    const int bnz = b.z1 - b.z0 + 1;
    const int dz = blockIdx.x * blockDim.x + threadIdx.x;
    if (dz >= bnz) return;
    long long idx = ((long long)(b.x0 + blockIdx.z) * ny + (b.y0 + blockIdx.y)) * nz + b.z0 + dz;
    double v[3] = {v0, v1, v2};
    for (int c = 0; c < comps; ++c) planes[c * n + idx] = (V)v[c];
}

// InitializeMomentumExchangeFunctional3D (bounceBackModels3D.hh:42-90): fluid
// directions of every momentum-exchange cell.  A neighbour outside a
// non-periodic domain is an envelope cell with the background dynamics,
// which counts as fluid.
__global__ void mebbMaskKernel(DevLattice L, uint32_t* out) {
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y, x = blockIdx.z;
    if (z >= L.nz) return;
    const long long idx = ((long long)x * L.ny + y) * L.nz + z;
    uint32_t m = 0;
    if (L.flags[idx] == K_MEBB) {
        Neighbourhood nb = neighbourhood(L, x, y, z);
        for (int i = 1; i < 19; ++i) {
            long long off;
            int pk = nb.move(i, +1, off) ? L.flags[idx + off] : K_BGK;
            if (pk != K_MEBB && pk != K_BB && pk != K_NODYN) m |= 1u << i;
        }
    }
    out[idx] = m;
}

// Per tile (row r, cells z0 .. z1-1 with z0 = t * kTileCells): bit 0 some
// cell of the tile is part of the lattice, bit 1 every cell from z0 - 1 to z1
// is (wrapping around a periodic z axis; beyond a non-periodic one nothing
// needs to be).
__global__ void tileLiveKernel(const uint8_t* flags, int rows, int nz, int tiles, int perZ, uint8_t* live) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)rows * tiles) return;
    const int r = (int)(i / tiles), t = (int)(i - (long long)r * tiles);
    const int z0 = t * kTileCells, z1 = min(z0 + kTileCells, nz);
    const uint8_t* f = flags + (long long)r * nz;
    bool any = false, all = true;
    for (int z = z0 - 1; z <= z1; ++z) {
        int zz = z;
        if (zz < 0 || zz >= nz) {
            if (!perZ) continue;
            zz = zz < 0 ? zz + nz : zz - nz;
        }
        const bool in = f[zz] != K_NONE;
        all &= in;
        if (z >= z0 && z < z1) any |= in;
    }
    live[i] = (uint8_t)((any ? 1 : 0) | (all ? 2 : 0));
}

// Per cell of the masked tiles: bit k set when the neighbour x + c_k is
// outside the lattice (its rows are interior rows: x and y moves stay inside;
// along z a periodic axis wraps and a non-periodic one's edge is the kernels'
// own domain-edge rule).
__global__ void tileMaskKernel(const uint8_t* flags, int ny, int nz, int perZ, const int4* tiles, int nTiles,
                               uint32_t* masks) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)nTiles * kTileCells) return;
    const int4 t = tiles[i / kTileCells];
    const int z = t.z + (int)(i % kTileCells);
    uint32_t m = 0;
    if (z < t.w) {
        for (int k = 1; k < 19; ++k) {
            int zz = z + cdir(k, 2);
            if (zz < 0 || zz >= nz) {
                if (!perZ) continue;
                zz = zz < 0 ? zz + nz : zz - nz;
            }
            const long long nb = ((long long)(t.x + cdir(k, 0)) * ny + (t.y + cdir(k, 1))) * nz + zz;
            if (flags[nb] == K_NONE) m |= 1u << k;
        }
    }
    masks[i] = m;
}

__global__ void kindMaskKernel(const uint8_t* flags, long long n, unsigned long long* mask) {
    unsigned long long m = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        int k = flags[i];
        m |= 1ull << (k < 63 ? k : 63);
    }
    for (int o = 16; o > 0; o >>= 1) m |= __shfl_down_sync(0xffffffffu, m, o);
    if ((threadIdx.x & 31) == 0 && m) atomicOr(mask, m);
}

// Block of coordinate p along an axis of n cells cut into b blocks by
// createRegularDistribution3D: the first n % b blocks are one cell longer.
__device__ __forceinline__ int regularBlock(int p, int n, int b) {
    const int q = n / b, r = n % b;
    return p < r * (q + 1) ? p / (q + 1) : r + (p - r * (q + 1)) / q;
}

// ComputeSparsityFunctional3D (offLattice/makeSparse3D.hh:47-76): a block is
// kept when some cell of its bulk has a non-zero field value.
__global__ void sparseKeepKernel(const int32_t* field, DevLattice L, int bx, int by, int bz, uint8_t* keep) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < L.n;
         idx += (long long)gridDim.x * blockDim.x) {
        if (field[idx] == 0) continue;
        const int z = (int)(idx % L.nz), y = (int)((idx / L.nz) % L.ny), x = (int)(idx / ((long long)L.ny * L.nz));
        keep[(regularBlock(x, L.nx, bx) * by + regularBlock(y, L.ny, by)) * bz + regularBlock(z, L.nz, bz)] = 1;
    }
}

// Cells of dropped blocks leave the lattice.
__global__ void sparseMarkKernel(DevLattice L, int bx, int by, int bz, const uint8_t* keep) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < L.n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int z = (int)(idx % L.nz), y = (int)((idx / L.nz) % L.ny), x = (int)(idx / ((long long)L.ny * L.nz));
        if (!keep[(regularBlock(x, L.nx, bx) * by + regularBlock(y, L.ny, by)) * bz + regularBlock(z, L.nz, bz)])
            const_cast<uint8_t*>(L.flags)[idx] = K_NONE;
    }
}

// Whether the edge / corner cell at (x, y, z) may read its neighbour one step
// along `axis`: inside the domain after the periodic wrap and part of the
// lattice, and -- for a
// density read -- not a cell whose populations the same pass rewrites.
__device__ bool surfaceReadOk(const DevLattice& L, int x, int y, int z, int axis, int step, int forbidFrom) {
    int p[3] = {x, y, z};
    const int n[3] = {L.nx, L.ny, L.nz};
    p[axis] += step;
    if (p[axis] < 0 || p[axis] >= n[axis]) {
        if (!L.per[axis] || n[axis] < 2) return false;
        p[axis] = p[axis] < 0 ? p[axis] + n[axis] : p[axis] - n[axis];
    }
    const int k = L.flags[((long long)p[0] * L.ny + p[1]) * L.nz + p[2]];
    if (k == K_NONE) return false;
    return !(forbidFrom >= 0 && k >= forbidFrom && k < K_NKINDS);
}

// Edge and corner cells (edges first) -- or, with out == nullptr, their
// counts -- and the lowest cell index whose finite differences cannot be
// taken (surfaceReadOk).
__global__ void surfaceListKernel(DevLattice L, int4* out, int edgeCap, int* counts, unsigned long long* bad) {
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < L.n;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k = L.flags[idx];
        if (!isSurface(k)) continue;
        const int z = (int)(idx % L.nz), y = (int)((idx / L.nz) % L.ny), x = (int)(idx / ((long long)L.ny * L.nz));
        bool ok = true;
        if (k < K_CORNER) {
            const int e = k - K_EDGE, plane = e / 4, d1 = (plane + 1) % 3, d2 = (plane + 2) % 3;
            const int n1 = (e & 2) ? 1 : -1, n2 = (e & 1) ? 1 : -1;
            ok = surfaceReadOk(L, x, y, z, plane, 1, -1) && surfaceReadOk(L, x, y, z, plane, -1, -1) &&
                 surfaceReadOk(L, x, y, z, d1, -n1, K_EDGE) && surfaceReadOk(L, x, y, z, d2, -n2, K_EDGE);
        } else {
            const int q = k - K_CORNER;
            ok = surfaceReadOk(L, x, y, z, 0, (q & 4) ? -1 : 1, K_CORNER) &&
                 surfaceReadOk(L, x, y, z, 1, (q & 2) ? -1 : 1, K_CORNER) &&
                 surfaceReadOk(L, x, y, z, 2, (q & 1) ? -1 : 1, K_CORNER);
        }
        if (!ok) atomicMin(bad, (unsigned long long)idx);
        const int which = k < K_CORNER ? 0 : 1;
        const int slot = atomicAdd(&counts[which], 1);
        if (out) out[which == 0 ? slot : edgeCap + slot] = make_int4(x, y, z, k);
    }
}

int launchBox(plbgpu_ctx* c) {
    c->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, PLBGPU_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    return PLBGPU_OK;
}

// Allocate the optional per-cell arrays the current kinds need.
int ensureAux(plbgpu_ctx* c, Domain* d, bool needBc, bool needForce, bool needMebb) {
    if (needBc && !d->bc) {
        CUDA_TRY(c, cudaMalloc(&d->bc, sizeof(double) * 3 * d->n));
        CUDA_TRY(c, cudaMemsetAsync(d->bc, 0, sizeof(double) * 3 * d->n, c->stream));
        d->deviceBytes += sizeof(double) * 3 * d->n;
    }
    if (needForce && !d->force) {
        size_t fs = d->precision == PLBGPU_FP64 ? sizeof(double) : sizeof(float);
        CUDA_TRY(c, cudaMalloc(&d->force, fs * 3 * d->n));
        CUDA_TRY(c, cudaMemsetAsync(d->force, 0, fs * 3 * d->n, c->stream));
        d->deviceBytes += fs * 3 * d->n;
    }
    if (needMebb && !d->mebb) {
        CUDA_TRY(c, cudaMalloc(&d->mebb, sizeof(uint32_t) * d->n));
        CUDA_TRY(c, cudaMemsetAsync(d->mebb, 0, sizeof(uint32_t) * d->n, c->stream));
        d->deviceBytes += sizeof(uint32_t) * d->n;
    }
    return PLBGPU_OK;
}

// Which kinds occur in the domain (bit k set for kind k).
int kindMask(plbgpu_ctx* c, Domain* d, unsigned long long* mask) {
    int rc = ensureStaging(c, 64);
    if (rc) return rc;
    unsigned long long* dm = static_cast<unsigned long long*>(c->staging);
    CUDA_TRY(c, cudaMemsetAsync(dm, 0, sizeof(unsigned long long), c->stream));
    kindMaskKernel<<<1024, 256, 0, c->stream>>>(d->flags, d->n, dm);
    if ((rc = launchBox(c))) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(mask, dm, sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return PLBGPU_OK;
}

// The tile lists of a sparse domain: tiles of up to kTileCells cells of a row
// whose 3x3 neighbourhood of rows is part of the lattice from one cell before
// the tile to one cell after it ("dense": the interior-row kernels step them,
// no neighbour falls outside); the other tiles of interior rows with a live
// cell ("masked": the one-cell row kernel, with each cell's mask of neighbours
// outside the lattice, which follow the domain-edge rule); the tiles of the
// domain's border rows with a live cell (the general kernel).  Tiles without
// live cells are left out.  Rebuilt when the kinds or the periodicity change.
int buildTileLists(plbgpu_ctx* c, Domain* d) {
    const int rows = d->nx * d->ny;
    const int tiles = (d->nz + kTileCells - 1) / kTileCells;
    const size_t nt = (size_t)rows * tiles;
    int rc = ensureStaging(c, nt);
    if (rc) return rc;
    uint8_t* dl = static_cast<uint8_t*>(c->staging);
    tileLiveKernel<<<(unsigned)((nt + 255) / 256), 256, 0, c->stream>>>(d->flags, rows, d->nz, tiles, d->per[2], dl);
    if ((rc = launchBox(c))) return rc;
    std::vector<uint8_t> live(nt);
    CUDA_TRY(c, cudaMemcpyAsync(live.data(), dl, nt, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    auto at = [&](int x, int y, int t) { return live[((size_t)x * d->ny + y) * tiles + t]; };
    std::vector<int4> dense, masked, general;
    for (int x = 0; x < d->nx; ++x)
        for (int y = 0; y < d->ny; ++y)
            for (int t = 0; t < tiles; ++t) {
                if (!(at(x, y, t) & 1)) continue;
                const bool interiorRow = x >= 1 && x <= d->nx - 2 && y >= 1 && y <= d->ny - 2;
                bool full = interiorRow;
                for (int dx = -1; dx <= 1 && full; ++dx)
                    for (int dy = -1; dy <= 1 && full; ++dy) full = (at(x + dx, y + dy, t) & 2) != 0;
                const int z0 = t * kTileCells, z1 = std::min(z0 + kTileCells, d->nz);
                (full ? dense : interiorRow ? masked : general).push_back(make_int4(x, y, z0, z1));
            }
    const int total = (int)(dense.size() + masked.size() + general.size());
    if (total > d->tileListCap) {
        if (d->tileLists) {
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            cudaFree(d->tileLists);
            d->deviceBytes -= sizeof(int4) * (size_t)d->tileListCap;
            d->tileLists = nullptr;
            d->tileListCap = 0;
        }
        CUDA_TRY(c, cudaMalloc(&d->tileLists, sizeof(int4) * (size_t)(total > 0 ? total : 1)));
        d->tileListCap = total > 0 ? total : 1;
        d->deviceBytes += sizeof(int4) * (size_t)d->tileListCap;
    }
    const int nd = (int)dense.size(), nm = (int)masked.size();
    dense.insert(dense.end(), masked.begin(), masked.end());
    dense.insert(dense.end(), general.begin(), general.end());
    if (total)
        CUDA_TRY(c, cudaMemcpyAsync(d->tileLists, dense.data(), sizeof(int4) * (size_t)total, cudaMemcpyHostToDevice,
                                    c->stream));
    if (nm > d->tileMaskCap) {
        if (d->tileMasks) {
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            cudaFree(d->tileMasks);
            d->deviceBytes -= sizeof(uint32_t) * kTileCells * (size_t)d->tileMaskCap;
            d->tileMasks = nullptr;
            d->tileMaskCap = 0;
        }
        CUDA_TRY(c, cudaMalloc(&d->tileMasks, sizeof(uint32_t) * kTileCells * (size_t)nm));
        d->tileMaskCap = nm;
        d->deviceBytes += sizeof(uint32_t) * kTileCells * (size_t)nm;
    }
    if (nm) {
        const long long cells = (long long)nm * kTileCells;
        tileMaskKernel<<<(unsigned)((cells + 255) / 256), 256, 0, c->stream>>>(d->flags, d->ny, d->nz, d->per[2],
                                                                            d->tileLists + nd, nm, d->tileMasks);
        if ((rc = launchBox(c))) return rc;
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    d->nDense = nd;
    d->nMasked = nm;
    d->nGeneral = (int)general.size();
    return PLBGPU_OK;
}

int syncKinds(plbgpu_ctx* c, Domain* d) {
    unsigned long long m = 0;
    int rc = kindMask(c, d, &m);
    if (rc) return rc;
    bool faces = false, surface = false;
    for (int k = K_REGVEL; k < K_NKINDS; ++k) faces |= (m >> k) & 1;
    for (int k = K_EDGE; k < K_NKINDS; ++k) surface |= (m >> k) & 1;
    d->hasSurface = surface;
    d->surfDirty = true;
    d->rowFacesDirty = true;
    d->sparse = (m >> 63) & 1;   // kinds >= 63: only K_NONE
    if (d->sparse && (rc = buildTileLists(c, d))) return rc;
    return ensureAux(c, d, faces, (m >> K_GUO) & 1, (m >> K_MEBB) & 1);
}

// Rebuild the edge / corner list, checking that every finite difference stays
// inside the domain.
int buildSurface(plbgpu_ctx* c, Domain* d) {
    d->surfDirty = false;
    d->nEdges = d->nCorners = 0;
    if (!d->hasSurface) return PLBGPU_OK;
    int rc = ensureStaging(c, 64);
    if (rc) return rc;
    int* counts = static_cast<int*>(c->staging);
    unsigned long long* bad = reinterpret_cast<unsigned long long*>(static_cast<char*>(c->staging) + 16);
    CUDA_TRY(c, cudaMemsetAsync(counts, 0, 2 * sizeof(int), c->stream));
    CUDA_TRY(c, cudaMemsetAsync(bad, 0xff, sizeof(unsigned long long), c->stream));
    surfaceListKernel<<<304, 256, 0, c->stream>>>(d->view(), nullptr, 0, counts, bad);
    if ((rc = launchBox(c))) return rc;
    int hc[2];
    unsigned long long hbad;
    CUDA_TRY(c, cudaMemcpyAsync(hc, counts, sizeof(hc), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(&hbad, bad, sizeof(hbad), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (hbad != ~0ull) {
        d->surfDirty = true;
        long long i = (long long)hbad;
        return fail(c, PLBGPU_ERR_ARG,
                    "edge/corner cell (%lld, %lld, %lld): its finite differences need neighbours inside the "
                    "domain, and a face or bulk cell (edges) or a non-corner cell (corners) inward along each normal",
                    i / ((long long)d->ny * d->nz), (i / d->nz) % d->ny, i % d->nz);
    }
    const int total = hc[0] + hc[1];
    if (total > d->surfCap) {
        if (d->surf) {
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            cudaFree(d->surf);
            d->deviceBytes -= sizeof(int4) * (size_t)d->surfCap;
            d->surf = nullptr;
            d->surfCap = 0;
        }
        CUDA_TRY(c, cudaMalloc(&d->surf, sizeof(int4) * (size_t)total));
        d->surfCap = total;
        d->deviceBytes += sizeof(int4) * (size_t)total;
    }
    CUDA_TRY(c, cudaMemsetAsync(counts, 0, 2 * sizeof(int), c->stream));
    surfaceListKernel<<<304, 256, 0, c->stream>>>(d->view(), d->surf, hc[0], counts, bad);
    if ((rc = launchBox(c))) return rc;
    d->nEdges = hc[0];
    d->nCorners = hc[1];
    return PLBGPU_OK;
}

// Steps per CUDA graph of a long collide_and_stream call (even: the graph
// ends on the parity it started on), and the replays that make capturing it
// worth while.
constexpr int kGraphSteps = 16;
constexpr int kGraphMinReplays = 2;

// Salt of the stochastically rounded stores of the step that follows
// `steps` steps.
unsigned stepSeed(long long steps) { return (unsigned)(steps * 0x9E3779B97F4A7C15ull >> 32); }

StepConsts consts(const Domain* d) {
    StepConsts s;
    // bgk_ma2_collision_base (dynamicsTemplates3D.h:2290-2293) with
    // t_0 = 1/3, t_1 = 1/18, t_4 = 1/36.
    s.omega = d->omega;
    s.one_m_omega = (double)1 - d->omega;
    s.t0_omega = ((double)1 / (double)3) * d->omega;
    s.t1_omega = ((double)1 / (double)18) * d->omega;
    s.t4_omega = ((double)1 / (double)36) * d->omega;
    s.invRho0 = (double)1 / d->rho0;
    s.pending = d->pending ? 1 : 0;
    s.seed = stepSeed(d->steps);
    s.external = 0;
    return s;
}

// The step kernels record a diverged state (a NaN or an infinity met by a
// statistics step) in the domain's device status word; report it once and
// clear it, so that the context stays usable (a new state can be sent).
int checkStatus(plbgpu_ctx* c, Domain* d) {
    unsigned st = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&st, d->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (st) {
        CUDA_TRY(c, cudaMemsetAsync(d->status, 0, sizeof(unsigned), c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        if (st & kStatusNonFinite)
            return fail(c, PLBGPU_ERR_STATE,
                        "non-finite populations (NaN or infinity) met by a statistics step: the run has diverged");
        return fail(c, PLBGPU_ERR_CUDA, "device status 0x%x", st);
    }
    return PLBGPU_OK;
}

// Complete pending faces in place so that the stored state is the
// reference's post-step state again.
int materialize(plbgpu_ctx* c, Domain* d) {
    if (!d->pending) return PLBGPU_OK;
    if (d->bc) {
        int n = launchers(d->precision).completeFaces(d->view(), d->odd, c->stream);
        c->launches += n - 1;
        int rc = launchBox(c);
        if (rc) return rc;
    }
    d->pending = false;
    return PLBGPU_OK;
}

// Face cells of interior rows (1 <= x <= nx-2, 1 <= y <= ny-2): counted into
// count[0] and, with out, listed (x, y, z, kind) in any order.
__global__ void rowFaceListKernel(const uint8_t* flags, int nx, int ny, int nz, int4* out, int cap, int* count) {
    const long long n = (long long)nx * ny * nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int k = flags[i];
        if (!isFace(k)) continue;
        const int z = (int)(i % nz), y = (int)((i / nz) % ny), x = (int)(i / ((long long)ny * nz));
        if (x < 1 || x > nx - 2 || y < 1 || y > ny - 2) continue;
        const int slot = atomicAdd(count, 1);
        if (out && slot < cap) out[slot] = make_int4(x, y, z, k);
    }
}

// The face list of the interior rows, for a dense FP64 domain whose steps use
// the interior-row kernels.  Only FP64 gains: a face cell's completion is a
// few hundred FP64 operations, which the warp of an interior row runs for its
// one face lane on the FP64 pipe (a lid-driven 64^3 cavity: 1431 MLUPS with
// completion in the row kernel, 2413 with the list); in FP32 the completion
// is cheap and the extra launch costs more on small domains (64^3: 23.9 against
// 18.1 GLUPS).  Sparse and thin domains complete in place.
int buildRowFaces(plbgpu_ctx* c, Domain* d) {
    d->rowFacesDirty = false;
    d->nRowFaces = 0;
    if (d->precision != PLBGPU_FP64 || d->sparse || !d->bc || d->nx < 3 || d->ny < 3) return PLBGPU_OK;
    int rc = ensureStaging(c, 16);
    if (rc) return rc;
    int* count = static_cast<int*>(c->staging);
    CUDA_TRY(c, cudaMemsetAsync(count, 0, sizeof(int), c->stream));
    rowFaceListKernel<<<1216, 256, 0, c->stream>>>(d->flags, d->nx, d->ny, d->nz, nullptr, 0, count);
    if ((rc = launchBox(c))) return rc;
    int n = 0;
    CUDA_TRY(c, cudaMemcpyAsync(&n, count, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (n == 0) return PLBGPU_OK;
    if (n > d->rowFaceCap) {
        if (d->rowFaces) {
            cudaFree(d->rowFaces);
            d->deviceBytes -= sizeof(int4) * (size_t)d->rowFaceCap;
            d->rowFaces = nullptr;
            d->rowFaceCap = 0;
        }
        CUDA_TRY(c, cudaMalloc(&d->rowFaces, sizeof(int4) * (size_t)n));
        d->rowFaceCap = n;
        d->deviceBytes += sizeof(int4) * (size_t)n;
    }
    CUDA_TRY(c, cudaMemsetAsync(count, 0, sizeof(int), c->stream));
    rowFaceListKernel<<<1216, 256, 0, c->stream>>>(d->flags, d->nx, d->ny, d->nz, d->rowFaces, n, count);
    if ((rc = launchBox(c))) return rc;
    d->nRowFaces = n;
    return PLBGPU_OK;
}

// Before a step whose faces are pending: complete the faces of interior rows
// from their list, and tell the interior-row kernels (v.rowFacesDone).
int preCompleteRowFaces(plbgpu_ctx* c, Domain* d, const StepConsts& k, DevLattice& v) {
    if (!k.pending || d->nRowFaces == 0) return PLBGPU_OK;
    int n = launchers(d->precision).completeFaceList(v, d->odd, d->rowFaces, d->nRowFaces, c->stream);
    if (n) {
        c->launches += n - 1;
        int rc = launchBox(c);
        if (rc) return rc;
    }
    v.rowFacesDone = 1;
    return PLBGPU_OK;
}

// The edge processors, then the corner processors, on the current state
// (OuterVelocityEdgeFunctional3D / OuterVelocityCornerFunctional3D, which
// setVelocityConditionOnBlockBoundaries adds after the faces:
// boundaryCondition3D.hh:65-163).
int finishSurface(plbgpu_ctx* c, Domain* d) {
    int rc;
    if (d->surfDirty && (rc = buildSurface(c, d))) return rc;
    if (d->nEdges + d->nCorners == 0) return PLBGPU_OK;
    ProfRange prof("dataProcessor", (unsigned long long)(d->nEdges + d->nCorners));
    const Launchers& L = launchers(d->precision);
    const int pending = d->pending && d->bc ? 1 : 0;
    const double invRho0 = (double)1 / d->rho0;
    int n = L.surface(d->view(), d->odd, d->surf, d->nEdges, pending, invRho0, d->bbRho, d->omega, c->stream);
    if (n) {
        c->launches += n - 1;
        if ((rc = launchBox(c))) return rc;
    }
    n = L.surface(d->view(), d->odd, d->surf + d->nEdges, d->nCorners, pending, invRho0, d->bbRho, d->omega,
                  c->stream);
    if (n) {
        c->launches += n - 1;
        if ((rc = launchBox(c))) return rc;
    }
    return PLBGPU_OK;
}

// The external rho-bar / j planes, allocated (zero) on first use.
int ensureExt(plbgpu_ctx* c, Domain* d) {
    if (d->ext) return PLBGPU_OK;
    size_t fs = d->precision == PLBGPU_FP64 ? sizeof(double) : sizeof(float);
    CUDA_TRY(c, cudaMalloc(&d->ext, fs * 4 * d->n));
    CUDA_TRY(c, cudaMemsetAsync(d->ext, 0, fs * 4 * d->n, c->stream));
    d->deviceBytes += fs * 4 * d->n;
    return PLBGPU_OK;
}

// Scatter (gather = 0) or gather a packed box of (rho-bar, jx, jy, jz) values.
int extBox(plbgpu_ctx* c, Domain* d, const Box& b, double* packed, int gather) {
    dim3 g = rowGrid(b.z1 - b.z0 + 1, b.y1 - b.y0 + 1, b.x1 - b.x0 + 1, 128);
    if (d->precision == PLBGPU_FP64)
        boxPlanesKernel<double, double><<<g, 128, 0, c->stream>>>(static_cast<double*>(d->ext), d->n, d->ny, d->nz,
                                                                   b, packed, 4, gather);
    else
        boxPlanesKernel<float, double><<<g, 128, 0, c->stream>>>(static_cast<float*>(d->ext), d->n, d->ny, d->nz, b,
                                                                  packed, 4, gather);
    return launchBox(c);
}

}  // namespace

// =================================================================== adjoint hooks

namespace plbgpu {

int domainAccess(plbgpu_ctx* c, int h, DomainAccess* out) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = materialize(c, d))) return rc;
    out->L = d->view();
    out->precision = d->precision;
    out->odd = d->odd;
    out->pending = d->pending;
    out->omega = d->omega;
    out->rho0 = d->rho0;
    out->bbRho = d->bbRho;
    out->stream = c->stream;
    out->adjointSlot = &d->adjoint;
    out->adjointFree = &d->adjointFree;
    out->launches = &c->launches;
    return PLBGPU_OK;
}

int domainFail(plbgpu_ctx* c, int code, const char* msg) { return fail(c, code, "%s", msg); }

cudaStream_t contextStream(plbgpu_ctx* c) { return c ? c->stream : nullptr; }

void countLaunches(plbgpu_ctx* c, int n) {
    if (c) c->launches += (unsigned long long)n;
}

int domainSurface(plbgpu_ctx* c, int h, const int4** cells, int* nEdges, int* nCorners) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = materialize(c, d))) return rc;
    if (d->surfDirty && (rc = buildSurface(c, d))) return rc;
    *cells = d->surf;
    *nEdges = d->nEdges;
    *nCorners = d->nCorners;
    return PLBGPU_OK;
}

void domainSetState(plbgpu_ctx* c, int h, bool odd, bool pending) {
    Domain* d;
    if (lookup(c, h, &d)) return;
    d->odd = odd;
    d->pending = pending;
    d->statsValid = false;
}

}  // namespace plbgpu

// =================================================================== C ABI

extern "C" {

int plbgpu_create(int device, plbgpu_ctx** out) {
    if (!out) return PLBGPU_ERR_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return PLBGPU_ERR_CUDA;
    if (device < 0 || device >= count) return PLBGPU_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return PLBGPU_ERR_CUDA;
    plbgpu_ctx* c = new (std::nothrow) plbgpu_ctx();
    if (!c) return PLBGPU_ERR_NOMEM;
    c->device = device;
    int pageable = 0;
    if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, device) == cudaSuccess)
        c->pageableAccess = pageable != 0;
    const char* staged = getenv("PLBGPU_STAGED_TRANSFERS");
    c->forceStaged = staged && staged[0] == '1';
    const char* rowKernel = getenv("PLBGPU_ROW_KERNEL");
    c->rowForm = !rowKernel                           ? 0
                 : strcmp(rowKernel, "cell") == 0     ? 1
                 : strcmp(rowKernel, "vec4") == 0     ? 2
                 : strcmp(rowKernel, "vec2") == 0     ? 3
                 : strcmp(rowKernel, "vec8") == 0     ? 4
                                                      : 0;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return PLBGPU_ERR_CUDA;
    }
    // The border rows' stream has the highest priority: submitted after the
    // interior kernel, its blocks take the first SM slots that free up
    // instead of waiting for the interior kernel's last wave.
    int leastPriority = 0, greatestPriority = 0;
    cudaDeviceGetStreamPriorityRange(&leastPriority, &greatestPriority);
    if (cudaStreamCreateWithPriority(&c->side.stream, cudaStreamNonBlocking, greatestPriority) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->side.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->side.join, cudaEventDisableTiming) != cudaSuccess) {
        if (c->side.stream) cudaStreamDestroy(c->side.stream);
        if (c->side.fork) cudaEventDestroy(c->side.fork);
        cudaStreamDestroy(c->stream);
        delete c;
        return PLBGPU_ERR_CUDA;
    }
    *out = c;
    return PLBGPU_OK;
}

int plbgpu_destroy(plbgpu_ctx* c) {
    if (!c) return PLBGPU_ERR_ARG;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    std::vector<int> hs;
    for (auto& kv : c->domains) hs.push_back(kv.first);
    for (int h : hs) plbgpu_remove_domain(c, h);
    if (c->staging) cudaFree(c->staging);
    if (c->xfer) {
        cudaStreamSynchronize(c->xfer);
        cudaStreamDestroy(c->xfer);
    }
    for (cudaEvent_t e : c->slabEvents) cudaEventDestroy(e);
    cudaStreamSynchronize(c->side.stream);
    cudaEventDestroy(c->side.fork);
    cudaEventDestroy(c->side.join);
    cudaStreamDestroy(c->side.stream);
    cudaStreamDestroy(c->stream);
    delete c;
    return PLBGPU_OK;
}

const char* plbgpu_last_error(const plbgpu_ctx* c) { return c ? c->lastError.c_str() : "null context"; }

int plbgpu_launch_count(const plbgpu_ctx* c, unsigned long long* count) {
    if (!c || !count) return PLBGPU_ERR_ARG;
    *count = c->launches;
    return PLBGPU_OK;
}

int plbgpu_get_stream(const plbgpu_ctx* c, void** stream) {
    if (!c || !stream) return PLBGPU_ERR_ARG;
    *stream = (void*)c->stream;
    return PLBGPU_OK;
}

int plbgpu_synchronize(plbgpu_ctx* c) {
    if (!c) return PLBGPU_ERR_ARG;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    for (auto& kv : c->domains) {
        int rc = checkStatus(c, kv.second.get());
        if (rc) return rc;
    }
    return PLBGPU_OK;
}

int plbgpu_add_domain(plbgpu_ctx* c, int nx, int ny, int nz, int precision, int* handle) {
    if (!c || !handle) return PLBGPU_ERR_ARG;
    // x and y index the grid's z and y dimensions (at most 65535 blocks each).
    if (nx < 1 || ny < 1 || nz < 1 || nx > 65535 || ny > 65535)
        return fail(c, PLBGPU_ERR_ARG, "domain extent %dx%dx%d (nx, ny must be in [1, 65535])", nx, ny, nz);
    if (precision < PLBGPU_FP64 || precision > PLBGPU_BF16_SR)
        return fail(c, PLBGPU_ERR_ARG, "unknown precision %d", precision);
    CUDA_TRY(c, cudaSetDevice(c->device));
    std::unique_ptr<Domain> d(new Domain());
    d->nx = nx; d->ny = ny; d->nz = nz;
    d->precision = precision;
    d->n = (long long)nx * ny * nz;
    // The interior kernels index cells with 32-bit integers.
    if (d->n >= (1LL << 31)) return fail(c, PLBGPU_ERR_ARG, "domain of %lld cells: split it below 2^31 cells", d->n);
    d->stride = (d->n + 127) / 128 * 128;   // every plane starts on a 256-byte boundary
    d->elemSize = elemSizeOf(precision);
    size_t popBytes = d->elemSize * 19 * (size_t)d->stride;
    size_t bytes = popBytes + (size_t)d->stride;
    CUDA_TRY(c, cudaMalloc(&d->arena, bytes));
    d->flags = static_cast<uint8_t*>(d->arena) + popBytes;
    d->deviceBytes = bytes;
    CUDA_TRY(c, cudaMemsetAsync(d->arena, 0, bytes, c->stream));   // f-bar = 0 (rest), all BGK
    CUDA_TRY(c, cudaMalloc(&d->stats, sizeof(StatsAcc) * kStatsSlots));
    CUDA_TRY(c, cudaMalloc(&d->status, sizeof(unsigned)));
    CUDA_TRY(c, cudaMemsetAsync(d->status, 0, sizeof(unsigned), c->stream));
    CUDA_TRY(c, cudaMalloc(&d->red, sizeof(ReduceAcc) * kStatsSlots));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    int h = c->nextHandle++;
    c->domains[h] = std::move(d);
    *handle = h;
    return PLBGPU_OK;
}

int plbgpu_remove_domain(plbgpu_ctx* c, int h) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    cudaStreamSynchronize(c->stream);
    cudaFree(d->arena);
    if (d->bc) cudaFree(d->bc);
    if (d->force) cudaFree(d->force);
    if (d->ext) cudaFree(d->ext);
    if (d->mebb) cudaFree(d->mebb);
    if (d->surf) cudaFree(d->surf);
    if (d->tileLists) cudaFree(d->tileLists);
    if (d->tileMasks) cudaFree(d->tileMasks);
    if (d->rowFaces) cudaFree(d->rowFaces);
    cudaFree(d->stats);
    cudaFree(d->status);
    cudaFree(d->red);
    if (d->adjoint && d->adjointFree) d->adjointFree(d->adjoint);
    c->domains.erase(h);
    return PLBGPU_OK;
}

int plbgpu_domain_info(plbgpu_ctx* c, int h, int* nx, int* ny, int* nz, int* precision,
                       unsigned long long* device_bytes) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (nx) *nx = d->nx;
    if (ny) *ny = d->ny;
    if (nz) *nz = d->nz;
    if (precision) *precision = d->precision;
    if (device_bytes) *device_bytes = d->deviceBytes;
    return PLBGPU_OK;
}

int plbgpu_set_periodicity(plbgpu_ctx* c, int h, int px, int py, int pz) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    // The stored AA state of an odd step depends on the neighbourhood: bring
    // it back to natural order first.
    if (d->odd) {
        std::vector<double> tmp((size_t)d->n * 19);
        if ((rc = plbgpu_receive(c, h, 0, d->nx - 1, 0, d->ny - 1, 0, d->nz - 1, tmp.data(), tmp.size()))) return rc;
        d->per[0] = px != 0; d->per[1] = py != 0; d->per[2] = pz != 0;
        d->odd = false;
        d->surfDirty = d->hasSurface;
        if (d->sparse && (rc = buildTileLists(c, d))) return rc;
        return plbgpu_send(c, h, 0, d->nx - 1, 0, d->ny - 1, 0, d->nz - 1, tmp.data(), tmp.size());
    }
    d->per[0] = px != 0; d->per[1] = py != 0; d->per[2] = pz != 0;
    d->surfDirty = d->hasSurface;
    if (d->sparse) return buildTileLists(c, d);   // the tiles at the z ends depend on the z periodicity
    return PLBGPU_OK;
}

int plbgpu_set_params(plbgpu_ctx* c, int h, double omega, double rho0, double bb_rho) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (!(rho0 != 0.0)) return fail(c, PLBGPU_ERR_ARG, "rho0 must be non-zero");
    d->omega = omega;
    d->rho0 = rho0;
    d->bbRho = bb_rho;
    return PLBGPU_OK;
}

}  // extern "C"

namespace {

// The data-processor record that the reference's boundary-condition
// instantiator integrates beside a face, edge or corner kind over a box
// (boundaryCondition/boundaryInstantiator3D.h): the wrapped local boundary
// functional of a face (regularized and Zou/He alike), the finite-difference
// processor of an external velocity edge or corner; data "dxScale dtScale "
// of a functional with the default scales (atomicBlock/
// dataProcessingFunctional3D.cpp:62-65), level 0, acting on block 0 (the
// lattice's global id in the saved description).
ProcessorRecord boundaryRecord(int kind, const Box& b) {
    ProcessorRecord r;
    if (isFace(kind)) {
        r.name = "WrappedLocalBoundary3D_%TD";
    } else if (kind >= K_EDGE && kind < K_CORNER) {
        const int e = kind - K_EDGE, plane = e / 4, n1 = (e & 2) ? 1 : -1, n2 = (e & 1) ? 1 : -1;
        r.name = "OuterVelocityEdge_%TD_" + std::to_string(plane) + "_" + std::to_string(n1) + "_" + std::to_string(n2);
    } else {
        const int e = kind - K_CORNER;
        r.name = std::string("OuterVelocityCorner3D_%TD_") + ((e & 4) ? "1" : "-1") + "_" + ((e & 2) ? "1" : "-1") +
                 "_" + ((e & 1) ? "1" : "-1");
    }
    r.data = "0 0 ";
    const long long dom[6] = {b.x0, b.x1, b.y0, b.y1, b.z0, b.z1};
    std::copy(dom, dom + 6, r.domain);
    r.blocks = {0};
    return r;
}

}  // namespace

extern "C" {

int plbgpu_add_boundary(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, int kind) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    if (!isFace(kind) && !isSurface(kind))
        return fail(c, PLBGPU_ERR_ARG, "kind %d is not a face, edge or corner kind", kind);
    if ((rc = plbgpu_define_dynamics(c, h, x0, x1, y0, y1, z0, z1, kind))) return rc;
    d->processors.push_back(boundaryRecord(kind, b));
    return PLBGPU_OK;
}

int plbgpu_add_processor(plbgpu_ctx* c, int h, const char* name, const long long* domain, const char* data,
                         long long level, const long long* blocks, int nblocks) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (!name || !*name || !domain || !data || nblocks < 0 || (nblocks > 0 && !blocks))
        return fail(c, PLBGPU_ERR_ARG, "processor record: null name, domain, data or blocks");
    for (const char* p = name; *p; ++p)
        if (*p == '<' || *p == '>' || *p == ' ' || *p == '\n')
            return fail(c, PLBGPU_ERR_ARG, "processor name '%s' is not an XML tag text", name);
    if (strchr(data, '<') || strchr(data, '>'))
        return fail(c, PLBGPU_ERR_ARG, "processor data may not hold '<' or '>'");
    ProcessorRecord r;
    r.name = name;
    r.data = data;
    std::copy(domain, domain + 6, r.domain);
    r.level = level;
    r.blocks.assign(blocks, blocks + nblocks);
    d->processors.push_back(r);
    return PLBGPU_OK;
}

int plbgpu_clear_processors(plbgpu_ctx* c, int h) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    d->processors.clear();
    return PLBGPU_OK;
}

int plbgpu_processor_count(plbgpu_ctx* c, int h, int* count) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (!count) return fail(c, PLBGPU_ERR_ARG, "null count");
    *count = (int)d->processors.size();
    return PLBGPU_OK;
}

int plbgpu_get_processor(plbgpu_ctx* c, int h, int i, char* name, size_t nameCap, long long* domain, char* data,
                         size_t dataCap, long long* level, long long* blocks, int blocksCap, int* nblocks) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (i < 0 || i >= (int)d->processors.size())
        return fail(c, PLBGPU_ERR_ARG, "processor %d of %zu", i, d->processors.size());
    const ProcessorRecord& r = d->processors[(size_t)i];
    if (!name || nameCap <= r.name.size() || !data || dataCap <= r.data.size())
        return fail(c, PLBGPU_ERR_ARG, "processor %d: name needs %zu bytes, data %zu", i, r.name.size() + 1,
                    r.data.size() + 1);
    if (nblocks) *nblocks = (int)r.blocks.size();
    if ((int)r.blocks.size() > blocksCap || (!blocks && !r.blocks.empty()))
        return fail(c, PLBGPU_ERR_ARG, "processor %d acts on %zu blocks", i, r.blocks.size());
    memcpy(name, r.name.c_str(), r.name.size() + 1);
    memcpy(data, r.data.c_str(), r.data.size() + 1);
    if (domain) std::copy(r.domain, r.domain + 6, domain);
    if (level) *level = r.level;
    if (!r.blocks.empty()) std::copy(r.blocks.begin(), r.blocks.end(), blocks);
    return PLBGPU_OK;
}

int plbgpu_define_dynamics(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, int kind) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    if (kind < 0 || kind >= K_NKINDS) return fail(c, PLBGPU_ERR_ARG, "unknown cell kind %d", kind);
    if ((rc = materialize(c, d))) return rc;
    fillKindsKernel<<<rowGrid(z1 - z0 + 1, y1 - y0 + 1, x1 - x0 + 1, 128), 128, 0, c->stream>>>(
        d->flags, d->ny, d->nz, b, (uint8_t)kind);
    if ((rc = launchBox(c))) return rc;
    return syncKinds(c, d);
}

int plbgpu_set_kinds(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, const uint8_t* kinds,
                     size_t n) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    long long cells = boxCells(b);
    if (!kinds || (long long)n != cells) return fail(c, PLBGPU_ERR_ARG, "kinds: %zu values for %lld cells", n, cells);
    for (size_t i = 0; i < n; ++i)
        if (kinds[i] >= K_NKINDS && kinds[i] != K_NONE) return fail(c, PLBGPU_ERR_ARG, "unknown cell kind %d", kinds[i]);
    if ((rc = materialize(c, d))) return rc;
    if ((rc = ensureStaging(c, n))) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->staging, kinds, n, cudaMemcpyHostToDevice, c->stream));
    boxPlanesKernel<uint8_t, uint8_t><<<rowGrid(z1 - z0 + 1, y1 - y0 + 1, x1 - x0 + 1, 128), 128, 0, c->stream>>>(
        d->flags, d->n, d->ny, d->nz, b, static_cast<uint8_t*>(c->staging), 1, 0);
    if ((rc = launchBox(c))) return rc;
    return syncKinds(c, d);
}

int plbgpu_set_velocity_condition_on_block_boundaries(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1,
                                                      int z0, int z1) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    if (x1 - x0 < 2 || y1 - y0 < 2 || z1 - z0 < 2)
        return fail(c, PLBGPU_ERR_ARG, "velocity box [%d,%d]x[%d,%d]x[%d,%d]: every extent must be >= 3", x0, x1,
                    y0, y1, z0, z1);
    const int lo[3] = {x0, y0, z0}, hi[3] = {x1, y1, z1};
    std::vector<uint8_t> kinds((size_t)boxCells(b));
    if ((rc = plbgpu_get_kinds(c, h, x0, x1, y0, y1, z0, z1, kinds.data(), kinds.size()))) return rc;   // interior kept
    for (int x = x0; x <= x1; ++x)
        for (int y = y0; y <= y1; ++y)
            for (int z = z0; z <= z1; ++z) {
                const int p[3] = {x, y, z};
                int side[3], nSides = 0;   // -1 low side, +1 high side, 0 inside
                for (int a = 0; a < 3; ++a) {
                    side[a] = p[a] == lo[a] ? -1 : (p[a] == hi[a] ? 1 : 0);
                    nSides += side[a] != 0;
                }
                size_t o = ((size_t)(x - x0) * (y1 - y0 + 1) + (y - y0)) * (z1 - z0 + 1) + (z - z0);
                int k;
                if (nSides == 0) {
                    continue;
                } else if (nSides == 1) {
                    int a = side[0] ? 0 : (side[1] ? 1 : 2);
                    k = K_REGVEL + 2 * a + (side[a] > 0);
                } else if (nSides == 2) {
                    int plane = !side[0] ? 0 : (!side[1] ? 1 : 2);
                    int n1 = side[(plane + 1) % 3], n2 = side[(plane + 2) % 3];
                    k = K_EDGE + 4 * plane + 2 * (n1 > 0) + (n2 > 0);
                } else {
                    k = K_CORNER + 4 * (side[0] > 0) + 2 * (side[1] > 0) + (side[2] > 0);
                }
                kinds[o] = (uint8_t)k;
            }
    if ((rc = plbgpu_set_kinds(c, h, x0, x1, y0, y1, z0, z1, kinds.data(), kinds.size()))) return rc;
    // the processors the reference integrates, in its order: six faces, twelve
    // edges (plane 0, 1, 2; normals NN, NP, PN, PP), eight corners (x, y, z
    // sides N before P, x slowest) (boundaryCondition/boundaryCondition3D.hh:65-163)
    auto piece = [&](int kind, const int (&side)[3]) {   // side: -1 low, +1 high, 0 the inner extent
        int l[3], u[3];
        for (int a = 0; a < 3; ++a) {
            l[a] = side[a] < 0 ? lo[a] : side[a] > 0 ? hi[a] : lo[a] + 1;
            u[a] = side[a] < 0 ? lo[a] : side[a] > 0 ? hi[a] : hi[a] - 1;
        }
        d->processors.push_back(boundaryRecord(kind, Box{l[0], u[0], l[1], u[1], l[2], u[2]}));
    };
    for (int a = 0; a < 3; ++a)
        for (int o = -1; o <= 1; o += 2) {
            int side[3] = {0, 0, 0};
            side[a] = o;
            piece(K_REGVEL + 2 * a + (o > 0), side);
        }
    for (int plane = 0; plane < 3; ++plane)
        for (int n1 = -1; n1 <= 1; n1 += 2)
            for (int n2 = -1; n2 <= 1; n2 += 2) {
                int side[3] = {0, 0, 0};
                side[(plane + 1) % 3] = n1;
                side[(plane + 2) % 3] = n2;
                piece(K_EDGE + 4 * plane + 2 * (n1 > 0) + (n2 > 0), side);
            }
    for (int e = 0; e < 8; ++e) {
        const int side[3] = {(e & 4) ? 1 : -1, (e & 2) ? 1 : -1, (e & 1) ? 1 : -1};
        piece(K_CORNER + e, side);
    }
    return PLBGPU_OK;
}

int plbgpu_select_sparse_blocks(plbgpu_ctx* c, int h, const int32_t* field, size_t n, int bx, int by, int bz,
                                uint8_t* keep, size_t nblocks) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (!field || (long long)n != d->n) return fail(c, PLBGPU_ERR_ARG, "sparse field: %zu values for %lld cells", n, d->n);
    if (bx < 1 || by < 1 || bz < 1 || bx > d->nx || by > d->ny || bz > d->nz)
        return fail(c, PLBGPU_ERR_ARG, "%dx%dx%d blocks for a %dx%dx%d domain", bx, by, bz, d->nx, d->ny, d->nz);
    const size_t nb = (size_t)bx * by * bz;
    if (keep && nblocks != nb) return fail(c, PLBGPU_ERR_ARG, "keep: %zu entries for %zu blocks", nblocks, nb);
    if ((rc = materialize(c, d))) return rc;
    const size_t fieldBytes = sizeof(int32_t) * (size_t)d->n;
    if ((rc = ensureStaging(c, fieldBytes + nb))) return rc;
    int32_t* df = static_cast<int32_t*>(c->staging);
    uint8_t* dk = static_cast<uint8_t*>(c->staging) + fieldBytes;
    CUDA_TRY(c, cudaMemcpyAsync(df, field, fieldBytes, cudaMemcpyHostToDevice, c->stream));
    CUDA_TRY(c, cudaMemsetAsync(dk, 0, nb, c->stream));
    sparseKeepKernel<<<1216, 256, 0, c->stream>>>(df, d->view(), bx, by, bz, dk);
    if ((rc = launchBox(c))) return rc;
    std::vector<uint8_t> hk(nb);
    CUDA_TRY(c, cudaMemcpyAsync(hk.data(), dk, nb, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    size_t kept = 0;
    for (uint8_t v : hk) kept += v;
    if (!kept) return fail(c, PLBGPU_ERR_ARG, "the sparse field is zero everywhere: no block would remain");
    sparseMarkKernel<<<1216, 256, 0, c->stream>>>(d->view(), bx, by, bz, dk);
    if ((rc = launchBox(c))) return rc;
    if (keep) memcpy(keep, hk.data(), nb);
    if ((rc = syncKinds(c, d))) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    d->statsValid = false;
    return PLBGPU_OK;
}

int plbgpu_get_kinds(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, uint8_t* kinds,
                     size_t n) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    long long cells = boxCells(b);
    if (!kinds || (long long)n != cells) return fail(c, PLBGPU_ERR_ARG, "kinds: %zu values for %lld cells", n, cells);
    if ((rc = ensureStaging(c, n))) return rc;
    boxPlanesKernel<uint8_t, uint8_t><<<rowGrid(z1 - z0 + 1, y1 - y0 + 1, x1 - x0 + 1, 128), 128, 0, c->stream>>>(
        d->flags, d->n, d->ny, d->nz, b, static_cast<uint8_t*>(c->staging), 1, 1);
    if ((rc = launchBox(c))) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(kinds, c->staging, n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return PLBGPU_OK;
}

namespace {

// Values for the face / force planes of a box.  comps = 3 (velocity, force) or
// 1 (density); `field` non-null = one set of values per cell.
int setPlanes(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, bool forcePlanes, int comps,
              const double* field, size_t n, double v0, double v1, double v2) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    long long cells = boxCells(b);
    if (field && (long long)n != cells * comps)
        return fail(c, PLBGPU_ERR_ARG, "expected %lld values, got %zu", cells * comps, n);
    if ((rc = materialize(c, d))) return rc;   // faces pending on old values complete with the old values
    if ((rc = ensureAux(c, d, !forcePlanes, forcePlanes, false))) return rc;
    dim3 g = rowGrid(z1 - z0 + 1, y1 - y0 + 1, x1 - x0 + 1, 128);
    bool f32 = forcePlanes && d->precision != PLBGPU_FP64;
    if (field) {
        if ((rc = ensureStaging(c, sizeof(double) * n))) return rc;
        CUDA_TRY(c, cudaMemcpyAsync(c->staging, field, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        double* src = static_cast<double*>(c->staging);
        if (f32)
            boxPlanesKernel<float, double><<<g, 128, 0, c->stream>>>(static_cast<float*>(d->force), d->n, d->ny, d->nz, b, src, comps, 0);
        else
            boxPlanesKernel<double, double><<<g, 128, 0, c->stream>>>(
                forcePlanes ? static_cast<double*>(d->force) : d->bc, d->n, d->ny, d->nz, b, src, comps, 0);
    } else {
        if (f32)
            boxPlanesConstKernel<float><<<g, 128, 0, c->stream>>>(static_cast<float*>(d->force), d->n, d->ny, d->nz, b, v0, v1, v2, comps);
        else
            boxPlanesConstKernel<double><<<g, 128, 0, c->stream>>>(
                forcePlanes ? static_cast<double*>(d->force) : d->bc, d->n, d->ny, d->nz, b, v0, v1, v2, comps);
    }
    if ((rc = launchBox(c))) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return PLBGPU_OK;
}

}  // namespace

int plbgpu_set_boundary_velocity(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, double ux,
                                 double uy, double uz) {
    return setPlanes(c, h, x0, x1, y0, y1, z0, z1, false, 3, nullptr, 0, ux, uy, uz);
}
int plbgpu_set_boundary_velocity_field(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1,
                                       const double* values, size_t n) {
    if (!values) return fail(c, PLBGPU_ERR_ARG, "null values");
    return setPlanes(c, h, x0, x1, y0, y1, z0, z1, false, 3, values, n, 0, 0, 0);
}
int plbgpu_set_boundary_density(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, double rho) {
    return setPlanes(c, h, x0, x1, y0, y1, z0, z1, false, 1, nullptr, 0, rho, 0, 0);
}
int plbgpu_set_boundary_density_field(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1,
                                      const double* values, size_t n) {
    if (!values) return fail(c, PLBGPU_ERR_ARG, "null values");
    return setPlanes(c, h, x0, x1, y0, y1, z0, z1, false, 1, values, n, 0, 0, 0);
}
int plbgpu_set_force(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, double fx, double fy,
                     double fz) {
    return setPlanes(c, h, x0, x1, y0, y1, z0, z1, true, 3, nullptr, 0, fx, fy, fz);
}
int plbgpu_set_force_field(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1,
                           const double* values, size_t n) {
    if (!values) return fail(c, PLBGPU_ERR_ARG, "null values");
    return setPlanes(c, h, x0, x1, y0, y1, z0, z1, true, 3, values, n, 0, 0, 0);
}

int plbgpu_initialize_momentum_exchange(plbgpu_ctx* c, int h) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = ensureAux(c, d, false, false, true))) return rc;
    mebbMaskKernel<<<rowGrid(d->nz, d->ny, d->nx, 128), 128, 0, c->stream>>>(d->view(), d->mebb);
    if ((rc = launchBox(c))) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return PLBGPU_OK;
}

namespace {
int equilibrium(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, const double* field, size_t n,
                double rho, double ux, double uy, double uz) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    long long cells = boxCells(b);
    if (field && (long long)n != 4 * cells) return fail(c, PLBGPU_ERR_ARG, "expected %lld values, got %zu", 4 * cells, n);
    if ((rc = materialize(c, d))) return rc;
    const double* src = nullptr;
    if (field) {
        if ((rc = ensureStaging(c, sizeof(double) * n))) return rc;
        CUDA_TRY(c, cudaMemcpyAsync(c->staging, field, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
        src = static_cast<const double*>(c->staging);
    }
    double cst[4] = {rho, ux, uy, uz};
    int k = launchers(d->precision).equilibrium(d->view(), d->odd, b, src, cst, (double)1 / d->rho0, c->stream);
    c->launches += k - 1;
    if ((rc = launchBox(c))) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    d->statsValid = false;
    return PLBGPU_OK;
}
}  // namespace

int plbgpu_initialize_at_equilibrium(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1,
                                     double rho, double ux, double uy, double uz) {
    return equilibrium(c, h, x0, x1, y0, y1, z0, z1, nullptr, 0, rho, ux, uy, uz);
}
int plbgpu_initialize_at_equilibrium_field(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1,
                                           const double* rho_u, size_t n) {
    if (!rho_u) return fail(c, PLBGPU_ERR_ARG, "null values");
    return equilibrium(c, h, x0, x1, y0, y1, z0, z1, rho_u, n, 0, 0, 0, 0);
}

int plbgpu_initialize(plbgpu_ctx* c, int h) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    // initialize() twice completes twice, like the reference.
    if ((rc = materialize(c, d))) return rc;
    d->pending = true;
    return finishSurface(c, d);
}

}  // extern "C"

namespace {

// plbgpu_send / plbgpu_receive for transfer records of B (double, or float
// for the single-precision co-processor form).
template <typename B>
int insertRecords(const Launchers& L, const DevLattice& v, bool odd, const Box& b, const B* in, cudaStream_t s) {
    if constexpr (sizeof(B) == sizeof(double)) return L.insert(v, odd, b, in, s);
    else return L.insertF32(v, odd, b, in, s);
}
template <typename B>
int extractRecords(const Launchers& L, const DevLattice& v, bool odd, const Box& b, int pending, B* out,
                   cudaStream_t s) {
    if constexpr (sizeof(B) == sizeof(double)) return L.extract(v, odd, b, pending, out, s);
    else return L.extractF32(v, odd, b, pending, out, s);
}

// The order of plbgpu_run_host's slab operations, host logic only.  The
// domain is cut into x-slabs.  In the in-place (AA) layout a cell's records,
// inserted at either parity, fill exactly the slots that the cell's next step
// reads and writes; a step of a cell touches slots that only the steps of its
// neighbours touch before and after it.  So slab j takes its first step once
// its own records are in, step s once slabs j - 1 .. j + 1 took step s - 1,
// and its records are final once slabs j - 1 .. j + 1 took the last step.
// The first steps run as a ramp behind the send (slab j - k takes step k as
// soon as slab j is in), the steps between as whole-domain steps, and the
// last steps as a ramp that finishes slab 0 first, each slab received as soon
// as it is final.
enum : int { kSlabSend = 0, kSlabStep = 1, kSlabReceive = 2, kWholeSteps = 3 };
struct SlabOp {
    int kind, slab, step;   // kWholeSteps: steps [slab, step) of the whole domain
};
struct RunHostPlan {
    int width = 0, nslab = 0, rHead = 0, rTail = 0;
    bool statsHead = false, statsTail = false;   // a ramp holds a statistics step
    std::vector<SlabOp> ops;
};

// nx >= 4, nsteps >= 2.  Steps per ramp: a transfer of the state (19 FP64
// values per cell over the host link) lasts about two FP64 steps and tens of
// steps of the narrower forms, but the copies share the SMs with the steps;
// on GB300 ramps of 2 FP64 steps (3 of the other forms) hid them best of 1 to
// 12.  A ramp holds at most one statistics step, which gathers into the
// domain's accumulator while the other steps of the ramp run.
RunHostPlan planRunHost(int nx, bool periodicX, int nsteps, int statsEvery, bool fp64) {
    RunHostPlan p;
    p.width = std::max(2, (nx + 15) / 16);
    p.nslab = (nx + p.width - 1) / p.width;
    const int S = p.nslab;
    auto statsAt = [&](int t) { return statsEvery > 0 && ((t + 1) % statsEvery == 0 || t == nsteps - 1); };
    auto statsIn = [&](int a, int b) {
        int k = 0;
        for (int t = a; t < b; ++t) k += statsAt(t) ? 1 : 0;
        return k;
    };
    const int rMax = fp64 ? 2 : 3;
    p.rTail = std::min(rMax, nsteps - 1);
    while (p.rTail > 1 && statsIn(nsteps - p.rTail, nsteps) > 1) --p.rTail;
    p.rHead = std::min(rMax, nsteps - p.rTail);
    while (p.rHead > 1 && statsIn(0, p.rHead) > 1) --p.rHead;
    p.statsHead = statsIn(0, p.rHead) > 0;
    p.statsTail = statsIn(nsteps - p.rTail, nsteps) > 0;
    std::vector<int> done(S, 0), target(S, p.rHead);
    std::vector<char> sent(S, 0), received(S, 0);
    auto nbr = [&](int j, int side) {
        const int q = j + side;
        if (q >= 0 && q < S) return q;
        return periodicX ? (q + S) % S : -1;
    };
    auto ready = [&](int j) {
        if (!sent[j] || done[j] >= target[j]) return false;
        for (int sd = -1; sd <= 1; sd += 2) {
            const int q = nbr(j, sd);
            if (q >= 0 && done[q] < done[j]) return false;
        }
        return true;
    };
    auto final_ = [&](int j) {
        if (done[j] < nsteps) return false;
        for (int sd = -1; sd <= 1; sd += 2) {
            const int q = nbr(j, sd);
            if (q >= 0 && done[q] < nsteps) return false;
        }
        return true;
    };
    // every ready step, the lowest (slab + steps since base) first and the
    // higher slab on ties: the diagonals of the ramps
    auto drain = [&](int base) {
        for (;;) {
            int best = -1;
            long long bestKey = 0;
            for (int j = 0; j < S; ++j) {
                if (!ready(j)) continue;
                const long long key = (long long)(j + done[j] - base) * (S + 1) + (S - j);
                if (best < 0 || key < bestKey) {
                    best = j;
                    bestKey = key;
                }
            }
            if (best < 0) return;
            p.ops.push_back({kSlabStep, best, done[best]});
            if (++done[best] < nsteps) continue;
            for (int sd = -1; sd <= 1; ++sd) {   // the slabs this step may have made final
                const int q = sd == 0 ? best : nbr(best, sd);
                if (q >= 0 && !received[q] && final_(q)) {
                    p.ops.push_back({kSlabReceive, q, nsteps});
                    received[q] = 1;
                }
            }
        }
    };
    for (int j = 0; j < S; ++j) {
        p.ops.push_back({kSlabSend, j, 0});
        sent[j] = 1;
        drain(0);
    }
    p.ops.push_back({kWholeSteps, p.rHead, nsteps - p.rTail});
    std::fill(done.begin(), done.end(), nsteps - p.rTail);
    std::fill(target.begin(), target.end(), nsteps);
    drain(nsteps - p.rTail);
    return p;
}

// A contiguous copy between the caller's buffer and a device staging slot,
// run by the SMs: few blocks, each thread with UNROLL vectors in flight, so
// that a small share of the SMs saturates the host link while the others
// keep stepping.  (Copy-engine copies of a page-locked buffer that has gone
// untouched by them for some tens of milliseconds were measured 7-15 times
// slower on GB300; loads and stores from the SMs were not.)
template <typename V, int UNROLL>
__global__ void __launch_bounds__(256) bulkCopyKernel(const V* __restrict__ src, V* __restrict__ dst, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + (UNROLL - 1) * stride < n; i += UNROLL * stride) {
        V v[UNROLL];
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) v[u] = src[i + u * stride];
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) dst[i + u * stride] = v[u];
    }
    for (; i < n; i += stride) dst[i] = src[i];
}

// One double of every 4 KB of a host buffer read and written back by the
// whole GPU: the first touch of a page after a long pause is slow, and many
// threads take those misses side by side, where the few blocks of
// bulkCopyKernel would take them one after another (an 80 MB slab copy then
// ran several times slower).
__global__ void touchPagesKernel(double* p, long long values) {
    const long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 512;
    if (i < values) {
        volatile double* q = p + i;
        *q = *q;
    }
}

// Blocks of bulkCopyKernel (640 KB in flight): on GB300 beside FP64 steps 20
// blocks hid the transfers best of 12 to 128.
constexpr int kBulkCopyBlocks = 20;

int bulkCopy(plbgpu_ctx* c, void* dst, const void* src, size_t bytes, cudaStream_t s) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) | bytes;
    if (a % 16 == 0)
        bulkCopyKernel<uint4, 8><<<kBulkCopyBlocks, 256, 0, s>>>(static_cast<const uint4*>(src),
                                                                static_cast<uint4*>(dst), (long long)(bytes / 16));
    else
        bulkCopyKernel<unsigned long long, 16><<<kBulkCopyBlocks, 256, 0, s>>>(
            static_cast<const unsigned long long*>(src), static_cast<unsigned long long*>(dst), (long long)(bytes / 8));
    return launchBox(c);
}

template <typename B>
int sendRecords(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, const B* buf, size_t n) {
    ProfRange prof("io");
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    long long cells = boxCells(b);
    if (!buf || (long long)n != 19 * cells) return fail(c, PLBGPU_ERR_ARG, "send: %zu values for %lld cells", n, cells);
    if ((rc = materialize(c, d))) return rc;
    const Launchers& L = launchers(d->precision);
    if (const void* dp = directPointer(c, buf)) {
        // one pass: the insert kernel reads the caller's buffer itself
        int k = insertRecords<B>(L, d->view(), d->odd, b, static_cast<const B*>(dp), c->stream);
        c->launches += k - 1;
        if ((rc = launchBox(c))) return rc;
    } else {
        size_t stage = 0;
        forEachChunk(b, [](const Box&, size_t) { return PLBGPU_OK; }, &stage);
        stage = stage / sizeof(double) * sizeof(B);
        if ((rc = ensureStaging(c, stage))) return rc;
        rc = forEachChunk(b, [&](const Box& s, size_t off) -> int {
            CUDA_TRY(c, cudaMemcpyAsync(c->staging, buf + off, sizeof(B) * 19 * (size_t)boxCells(s),
                                        cudaMemcpyHostToDevice, c->stream));
            int k = insertRecords<B>(L, d->view(), d->odd, s, static_cast<const B*>(c->staging), c->stream);
            c->launches += k - 1;
            return launchBox(c);
        }, &stage);
        if (rc) return rc;
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    d->statsValid = false;
    return PLBGPU_OK;
}

template <typename B>
int receiveRecords(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, B* buf, size_t n) {
    ProfRange prof("io");
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    long long cells = boxCells(b);
    if (!buf || (long long)n != 19 * cells) return fail(c, PLBGPU_ERR_ARG, "receive: %zu values for %lld cells", n, cells);
    if ((rc = checkStatus(c, d))) return rc;
    const Launchers& L = launchers(d->precision);
    const int pending = d->pending && d->bc ? 1 : 0;
    if (const void* dp = directPointer(c, buf)) {
        // one pass: the extract kernel writes the caller's buffer itself
        int k = extractRecords<B>(L, d->view(), d->odd, b, pending, static_cast<B*>(const_cast<void*>(dp)), c->stream);
        c->launches += k - 1;
        if ((rc = launchBox(c))) return rc;
    } else {
        size_t stage = 0;
        forEachChunk(b, [](const Box&, size_t) { return PLBGPU_OK; }, &stage);
        stage = stage / sizeof(double) * sizeof(B);
        if ((rc = ensureStaging(c, stage))) return rc;
        rc = forEachChunk(b, [&](const Box& s, size_t off) -> int {
            int k = extractRecords<B>(L, d->view(), d->odd, s, pending, static_cast<B*>(c->staging), c->stream);
            c->launches += k - 1;
            int r = launchBox(c);
            if (r) return r;
            CUDA_TRY(c, cudaMemcpyAsync(buf + off, c->staging, sizeof(B) * 19 * (size_t)boxCells(s),
                                        cudaMemcpyDeviceToHost, c->stream));
            return PLBGPU_OK;
        }, &stage);
        if (rc) return rc;
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return PLBGPU_OK;
}

}  // namespace

extern "C" {

int plbgpu_send(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, const double* buf, size_t n) {
    return sendRecords<double>(c, h, x0, x1, y0, y1, z0, z1, buf, n);
}
int plbgpu_receive(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, double* buf, size_t n) {
    return receiveRecords<double>(c, h, x0, x1, y0, y1, z0, z1, buf, n);
}
int plbgpu_send_f32(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, const float* buf, size_t n) {
    return sendRecords<float>(c, h, x0, x1, y0, y1, z0, z1, buf, n);
}
int plbgpu_receive_f32(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, float* buf, size_t n) {
    return receiveRecords<float>(c, h, x0, x1, y0, y1, z0, z1, buf, n);
}

int plbgpu_collide_and_stream(plbgpu_ctx* c, int h, int nsteps, int collect_stats) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (nsteps < 0) return fail(c, PLBGPU_ERR_ARG, "nsteps %d", nsteps);
    if (nsteps == 0) return PLBGPU_OK;
    ProfRange prof("cycle", (unsigned long long)nsteps);
    const Launchers& L = launchers(d->precision);
    const bool hasFaces = d->bc != nullptr;
    if (d->surfDirty && (rc = buildSurface(c, d))) return rc;
    if (d->rowFacesDirty && (rc = buildRowFaces(c, d))) return rc;
    auto stepOnce = [&](bool stats) -> int {
        ProfRange step("collStream", (unsigned long long)d->n);
        if (stats) CUDA_TRY(c, cudaMemsetAsync(d->stats, 0, sizeof(StatsAcc) * kStatsSlots, c->stream));
        StepConsts k = consts(d);
        DevLattice v = d->view();
        v.rowForm = c->rowForm;
        int pr = preCompleteRowFaces(c, d, k, v);
        if (pr) return pr;
        int nl = L.step(v, d->odd, stats, k, d->stats, c->stream, &c->side);
        c->launches += nl - 1;
        int r = launchBox(c);
        if (r) return r;
        d->odd = !d->odd;
        d->pending = hasFaces;
        d->steps += 1;
        return finishSurface(c, d);
    };
    int s = 0;
    // The first step may complete faces lazily and the last may gather
    // statistics; the steps between repeat the same launches every two steps,
    // so a long run replays them from a CUDA graph of kGraphSteps steps
    // (fewer host launches and no stream-event round trips between the
    // interior and border kernels).  Stochastic rounding draws a new seed
    // every step and keeps the plain launches.
    if ((rc = stepOnce(collect_stats && nsteps == 1))) return rc;
    ++s;
    const int last = nsteps - (collect_stats ? 1 : 0);   // steps [s, last) gather nothing
    const int reps = (last - s) / kGraphSteps;
    if (reps >= kGraphMinReplays && d->precision != PLBGPU_BF16_SR) {
        const long long launches0 = c->launches;
        const bool odd0 = d->odd, pending0 = d->pending;
        const long long steps0 = d->steps;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        bool captured = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (captured) {
            for (int g = 0; g < kGraphSteps && rc == PLBGPU_OK; ++g) rc = stepOnce(false);
            captured = cudaStreamEndCapture(c->stream, &graph) == cudaSuccess && rc == PLBGPU_OK &&
                       cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
        }
        const long long perGraph = c->launches - launches0;
        // the capture only recorded the launches: the domain is where it was
        d->odd = odd0;
        d->pending = pending0;
        d->steps = steps0;
        c->launches = launches0;
        rc = PLBGPU_OK;
        (void)cudaGetLastError();
        if (captured) {
            for (int r = 0; r < reps && rc == PLBGPU_OK; ++r)
                if (cudaGraphLaunch(exec, c->stream) != cudaSuccess) rc = fail(c, PLBGPU_ERR_CUDA, "graph launch failed");
            if (rc == PLBGPU_OK) {
                s += reps * kGraphSteps;
                d->steps += (long long)reps * kGraphSteps;
                d->odd = (kGraphSteps % 2) ? !odd0 : odd0;
                d->pending = hasFaces;
                c->launches += perGraph * reps;
            }
        }
        if (exec) cudaGraphExecDestroy(exec);   // freed when the launches finish
        if (graph) cudaGraphDestroy(graph);
        if (rc) return rc;
    }
    for (; s < nsteps; ++s)
        if ((rc = stepOnce(collect_stats && s == nsteps - 1))) return rc;
    if (collect_stats) d->statsValid = true;
    return PLBGPU_OK;
}

int plbgpu_get_stats(plbgpu_ctx* c, int h, double out[7]) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (!out) return PLBGPU_ERR_ARG;
    if (!d->statsValid) return fail(c, PLBGPU_ERR_STATE, "no step has gathered statistics since the last change");
    if ((rc = checkStatus(c, d))) return rc;
    StatsAcc slots[kStatsSlots];
    CUDA_TRY(c, cudaMemcpyAsync(slots, d->stats, sizeof(slots), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    StatsAcc a = {0., 0., 0ull, 0ull, {0., 0., 0.}, 0.};
    for (const StatsAcc& s : slots) {
        a.sumRhoBar += s.sumRhoBar;
        a.sumUSqr += s.sumUSqr;
        a.count += s.count;
        a.maxBits = s.maxBits > a.maxBits ? s.maxBits : a.maxBits;
        for (int k = 0; k < 3; ++k) a.drag[k] += s.drag[k];
    }
    double cnt = (double)a.count;
    double mx;
    memcpy(&mx, &a.maxBits, sizeof(double));
    out[0] = a.count ? a.sumRhoBar / cnt : 0.;
    out[1] = a.count ? a.sumUSqr / cnt : 0.;
    out[2] = a.count ? mx : -1.79769313486231570815e+308;
    out[3] = a.drag[0];
    out[4] = a.drag[1];
    out[5] = a.drag[2];
    out[6] = cnt;
    return PLBGPU_OK;
}

int plbgpu_run_host(plbgpu_ctx* c, int h, const double* in, double* out, size_t n, int nsteps, int stats_every,
                    double* stats, size_t nstats) {
    ProfRange prof("cycle", (unsigned long long)(nsteps > 0 ? nsteps : 0));
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (!in || !out || (long long)n != 19 * d->n)
        return fail(c, PLBGPU_ERR_ARG, "run_host: %zu values for %lld cells", n, d->n);
    if (nsteps < 1 || stats_every < 0) return fail(c, PLBGPU_ERR_ARG, "run_host: nsteps %d, stats_every %d", nsteps,
                                                   stats_every);
    const int nrec = stats_every > 0 ? (nsteps + stats_every - 1) / stats_every : 0;
    if (nrec && (!stats || nstats < (size_t)7 * nrec))
        return fail(c, PLBGPU_ERR_ARG, "run_host: %d statistics records need %d doubles", nrec, 7 * nrec);
    auto statsAt = [&](int t) { return stats_every > 0 && ((t + 1) % stats_every == 0 || t == nsteps - 1); };
    int rec = 0;
    auto saveStats = [&]() { return plbgpu_get_stats(c, h, stats + 7 * rec++); };
    // steps [t, end) with the statistics records they owe, through the ordinary step call
    auto steps = [&](int t, int end) -> int {
        while (t < end) {
            int next = t;
            while (next < end && !statsAt(next)) ++next;
            if (next == end) return plbgpu_collide_and_stream(c, h, end - t, 0);
            int r = plbgpu_collide_and_stream(c, h, next - t + 1, 1);
            if (r || (r = saveStats())) return r;
            t = next + 1;
        }
        return PLBGPU_OK;
    };
    const int nx = d->nx, ny = d->ny, nz = d->nz;
    if ((rc = materialize(c, d))) return rc;
    if (d->surfDirty && (rc = buildSurface(c, d))) return rc;
    // The pipelined transfers are SM copies of the caller's buffers, which
    // the GPU must address directly (device or pinned memory, or any host
    // memory on a GB300).  Stochastically rounded BF16 draws its random bits
    // per kernel form (the paired stores hash one address for two slots):
    // slab steps would round differently from whole steps, so that form
    // steps in sequence.
    const double* din = static_cast<const double*>(directPointer(c, in));
    double* dout = static_cast<double*>(const_cast<void*>(directPointer(c, out)));
    const bool pipe = din && dout && !d->sparse && d->nEdges + d->nCorners == 0 && nsteps >= 2 && nx >= 4 &&
                      ny >= 3 && 2 * ny + 2 * nx <= 65535 && d->precision != PLBGPU_BF16_SR && c->side.stream;
    if (!pipe) {   // the three calls in sequence
        if ((rc = plbgpu_send(c, h, 0, nx - 1, 0, ny - 1, 0, nz - 1, in, n))) return rc;
        if ((rc = steps(0, nsteps))) return rc;
        return plbgpu_receive(c, h, 0, nx - 1, 0, ny - 1, 0, nz - 1, out, n);
    }
    const RunHostPlan plan = planRunHost(nx, d->per[0] != 0, nsteps, stats_every, d->precision == PLBGPU_FP64);
    const int width = plan.width, nslab = plan.nslab;
    while ((int)c->slabEvents.size() < 4 * nslab + 1) {
        cudaEvent_t e;
        CUDA_TRY(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->slabEvents.push_back(e);
    }
    if (!c->xfer) {   // the copies' blocks take the first SM slots that free up
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        CUDA_TRY(c, cudaStreamCreateWithPriority(&c->xfer, cudaStreamNonBlocking, greatest));
    }
    cudaEvent_t* copiedEv = c->slabEvents.data();   // slab j's records copied into the staging slot
    cudaEvent_t* insertedEv = copiedEv + nslab;     // ... inserted: the slot is free
    cudaEvent_t* extractedEv = insertedEv + nslab;  // the m-th slab received extracted into its slot
    cudaEvent_t* sentBackEv = extractedEv + nslab;  // ... copied out: the slot is free
    cudaEvent_t forkEv = c->slabEvents[4 * nslab];
    // staging: a ring of slab-sized slots between the copies and the kernels
    const int nSlots = std::min(4, nslab);
    const size_t slabValues = (size_t)width * ny * nz * 19;
    if ((rc = ensureStaging(c, sizeof(double) * slabValues * nSlots))) return rc;
    auto slot = [&](int m) { return static_cast<double*>(c->staging) + (size_t)(m % nSlots) * slabValues; };
    const Launchers& L = launchers(d->precision);
    const bool hasFaces = d->bc != nullptr;
    cudaStream_t xs = c->xfer;
    auto x0of = [&](int j) { return j * width; };
    auto x1of = [&](int j) { return std::min(nx - 1, j * width + width - 1); };
    auto records = [&](int j) { return (size_t)x0of(j) * ny * nz * 19; };
    auto bytesOf = [&](int j) { return sizeof(double) * (size_t)(x1of(j) - x0of(j) + 1) * ny * nz * 19; };
    auto box = [&](int j) { return Box{x0of(j), x1of(j), 0, ny - 1, 0, nz - 1}; };
    const bool odd0 = d->odd, pending0 = d->pending;
    const long long steps0 = d->steps;
    DevLattice v = d->view();
    v.rowForm = c->rowForm;
    int nSent = 0, nReceived = 0;
    // slab j's records copied into the next slot (the copy runs up to nSlots
    // slabs ahead of the inserts), then inserted on the step stream
    auto send = [&](int j) -> int {
        const int m = nSent++;
        if (m >= nSlots) CUDA_TRY(c, cudaStreamWaitEvent(xs, insertedEv[m - nSlots], 0));
        int r = bulkCopy(c, slot(m), din + records(j), bytesOf(j), xs);
        if (r) return r;
        CUDA_TRY(c, cudaEventRecord(copiedEv[m], xs));
        CUDA_TRY(c, cudaStreamWaitEvent(c->stream, copiedEv[m], 0));
        const int nl = insertRecords<double>(L, v, odd0, box(j), slot(m), c->stream);
        c->launches += nl - 1;
        if ((r = launchBox(c))) return r;
        CUDA_TRY(c, cudaEventRecord(insertedEv[m], c->stream));
        return PLBGPU_OK;
    };
    // slab j's final records extracted into the next slot on the step stream,
    // then copied out behind the steps that follow
    auto receive = [&](int j) -> int {
        const int m = nReceived++;
        if (m >= nSlots) CUDA_TRY(c, cudaStreamWaitEvent(c->stream, sentBackEv[m - nSlots], 0));
        const int nl = extractRecords<double>(L, v, odd0 ^ (nsteps & 1), box(j), hasFaces ? 1 : 0, slot(m),
                                              c->stream);
        c->launches += nl - 1;
        int r = launchBox(c);
        if (r) return r;
        CUDA_TRY(c, cudaEventRecord(extractedEv[m], c->stream));
        CUDA_TRY(c, cudaStreamWaitEvent(xs, extractedEv[m], 0));
        if ((r = bulkCopy(c, dout + records(j), slot(m), bytesOf(j), xs))) return r;
        CUDA_TRY(c, cudaEventRecord(sentBackEv[m], xs));
        return PLBGPU_OK;
    };
    auto stepSlab = [&](int j, int t) -> int {
        StepConsts k = consts(d);
        k.pending = (t == 0 ? pending0 : hasFaces) ? 1 : 0;
        k.seed = stepSeed(steps0 + t);
        const int nl = L.slabStep(v, odd0 ^ (t & 1), statsAt(t), k, d->stats, x0of(j), x1of(j), c->stream, &c->side);
        c->launches += nl - 1;
        return launchBox(c);
    };
    auto settle = [&](int t1, bool gathered) -> int {
        d->odd = odd0 ^ (t1 & 1);
        d->pending = hasFaces;
        d->steps = steps0 + t1;
        if (gathered) d->statsValid = true;
        int r = finishSurface(c, d);
        if (r || !gathered) return r;
        return saveStats();
    };
    {
        ProfRange io("io");
        if (plan.statsHead) CUDA_TRY(c, cudaMemsetAsync(d->stats, 0, sizeof(StatsAcc) * kStatsSlots, c->stream));
        CUDA_TRY(c, cudaEventRecord(forkEv, c->stream));
        CUDA_TRY(c, cudaStreamWaitEvent(xs, forkEv, 0));
        for (const SlabOp& op : plan.ops) {
            switch (op.kind) {
            case kSlabSend: rc = send(op.slab); break;
            case kSlabStep: rc = stepSlab(op.slab, op.step); break;
            case kSlabReceive: rc = receive(op.slab); break;
            default:   // the ramp behind the send is done: the steps between, then the closing ramp
                if ((rc = settle(plan.rHead, plan.statsHead))) return rc;
                if ((rc = steps(op.slab, op.step))) return rc;
                {   // the pages of `out` touched beside the first steps of the closing ramp
                    // (the send has read `in`, which may be `out`, before the steps between)
                    CUDA_TRY(c, cudaEventRecord(forkEv, c->stream));
                    CUDA_TRY(c, cudaStreamWaitEvent(xs, forkEv, 0));
                    const long long values = (long long)n, pages = (values + 511) / 512;
                    touchPagesKernel<<<(unsigned)((pages + 255) / 256), 256, 0, xs>>>(dout, values);
                    if ((rc = launchBox(c))) return rc;
                }
                if (plan.statsTail)
                    CUDA_TRY(c, cudaMemsetAsync(d->stats, 0, sizeof(StatsAcc) * kStatsSlots, c->stream));
                break;
            }
            if (rc) return rc;
        }
        if (nSent != nslab || nReceived != nslab)
            return fail(c, PLBGPU_ERR_STATE, "run_host: %d slabs sent and %d received of %d", nSent, nReceived,
                        nslab);
        CUDA_TRY(c, cudaStreamSynchronize(xs));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        if ((rc = settle(nsteps, plan.statsTail))) return rc;
    }
    return checkStatus(c, d);
}

int plbgpu_run_host_plan(int nx, int periodic_x, int nsteps, int stats_every, int precision, int* slab_width,
                         int* ops, size_t cap, size_t* count) {
    if (nx < 4 || nsteps < 2 || stats_every < 0 || precision < PLBGPU_FP64 || precision > PLBGPU_BF16_SR || !count)
        return PLBGPU_ERR_ARG;
    const RunHostPlan plan = planRunHost(nx, periodic_x != 0, nsteps, stats_every, precision == PLBGPU_FP64);
    *count = plan.ops.size();
    if (slab_width) *slab_width = plan.width;
    if (!ops) return PLBGPU_OK;
    if (cap < 3 * plan.ops.size()) return PLBGPU_ERR_ARG;
    for (size_t i = 0; i < plan.ops.size(); ++i) {
        ops[3 * i] = plan.ops[i].kind;
        ops[3 * i + 1] = plan.ops[i].slab;
        ops[3 * i + 2] = plan.ops[i].step;
    }
    return PLBGPU_OK;
}

int plbgpu_reduce(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, double* avg_energy,
                  double* avg_density) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    CUDA_TRY(c, cudaMemsetAsync(d->red, 0, sizeof(ReduceAcc) * kStatsSlots, c->stream));
    int k = launchers(d->precision).reduce(d->view(), d->odd, b, d->pending && d->bc ? 1 : 0, (double)1 / d->rho0,
                                           d->bbRho, d->red, c->stream);
    c->launches += k - 1;
    if ((rc = launchBox(c))) return rc;
    ReduceAcc slots[kStatsSlots];
    CUDA_TRY(c, cudaMemcpyAsync(slots, d->red, sizeof(slots), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    ReduceAcc a = {0., 0., 0ull};
    for (const ReduceAcc& s : slots) {
        a.sumEnergy += s.sumEnergy;
        a.sumRhoBar += s.sumRhoBar;
        a.cells += s.cells;
    }
    // computeAverage* over the cells of the lattice in the box (a sparse
    // domain's kept blocks)
    double cells = (double)a.cells;
    if (avg_energy) *avg_energy = a.sumEnergy / (double)2 / cells;
    if (avg_density) *avg_density = a.sumRhoBar / cells + (double)1;
    return PLBGPU_OK;
}

namespace {
int field(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, int what, double* out, size_t n) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    long long cells = boxCells(b);
    const int comps = what == 0 ? 3 : 1;
    if (!out || (long long)n != comps * cells)
        return fail(c, PLBGPU_ERR_ARG, "expected %lld values, got %zu", comps * cells, n);
    if ((rc = ensureStaging(c, sizeof(double) * n))) return rc;
    int k = launchers(d->precision).field(d->view(), d->odd, b, d->pending && d->bc ? 1 : 0, (double)1 / d->rho0,
                                          d->bbRho, what, static_cast<double*>(c->staging), c->stream);
    c->launches += k - 1;
    if ((rc = launchBox(c))) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(out, c->staging, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return PLBGPU_OK;
}
}  // namespace

int plbgpu_compute_velocity(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, double* out,
                            size_t n) {
    return field(c, h, x0, x1, y0, y1, z0, z1, 0, out, n);
}

int plbgpu_compute_density(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, double* out,
                           size_t n) {
    return field(c, h, x0, x1, y0, y1, z0, z1, 1, out, n);
}

int plbgpu_compute_rhobar_j(plbgpu_ctx* c, int h) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = ensureExt(c, d))) return rc;
    int n = launchers(d->precision).rhoBarJ(d->view(), d->odd, d->pending && d->bc ? 1 : 0, d->bbRho, c->stream);
    c->launches += n - 1;
    return launchBox(c);
}

int plbgpu_set_rhobar_j(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, const double* values,
                        size_t n) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    long long cells = boxCells(b);
    if (!values || (long long)n != 4 * cells)
        return fail(c, PLBGPU_ERR_ARG, "rho-bar/j: %zu values for %lld cells (4 per cell)", n, cells);
    if ((rc = ensureExt(c, d))) return rc;
    if ((rc = ensureStaging(c, sizeof(double) * n))) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(c->staging, values, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    if ((rc = extBox(c, d, b, static_cast<double*>(c->staging), 0))) return rc;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return PLBGPU_OK;
}

int plbgpu_get_rhobar_j(plbgpu_ctx* c, int h, int x0, int x1, int y0, int y1, int z0, int z1, double* out,
                        size_t n) {
    Domain* d;
    Box b;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if ((rc = checkBox(c, d, x0, x1, y0, y1, z0, z1, &b))) return rc;
    long long cells = boxCells(b);
    if (!out || (long long)n != 4 * cells)
        return fail(c, PLBGPU_ERR_ARG, "rho-bar/j: %zu values for %lld cells (4 per cell)", n, cells);
    if (!d->ext) return fail(c, PLBGPU_ERR_STATE, "no rho-bar/j fields yet");
    if ((rc = ensureStaging(c, sizeof(double) * n))) return rc;
    if ((rc = extBox(c, d, b, static_cast<double*>(c->staging), 1))) return rc;
    CUDA_TRY(c, cudaMemcpyAsync(out, c->staging, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return PLBGPU_OK;
}

int plbgpu_collide_and_stream_external(plbgpu_ctx* c, int h, int nsteps, int recompute, int collect_stats) {
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (nsteps < 0) return fail(c, PLBGPU_ERR_ARG, "nsteps %d", nsteps);
    if (!d->ext)
        return fail(c, PLBGPU_ERR_STATE,
                    "no rho-bar/j fields: call plbgpu_compute_rhobar_j or plbgpu_set_rhobar_j first");
    if (nsteps == 0) return PLBGPU_OK;
    const Launchers& L = launchers(d->precision);
    bool hasFaces = d->bc != nullptr;
    if (d->surfDirty && (rc = buildSurface(c, d))) return rc;
    if (d->rowFacesDirty && (rc = buildRowFaces(c, d))) return rc;
    for (int s = 0; s < nsteps; ++s) {
        bool stats = collect_stats && s == nsteps - 1;
        if (stats) CUDA_TRY(c, cudaMemsetAsync(d->stats, 0, sizeof(StatsAcc) * kStatsSlots, c->stream));
        StepConsts k = consts(d);
        k.external = 1;
        DevLattice v = d->view();
        v.rowForm = c->rowForm;
        if ((rc = preCompleteRowFaces(c, d, k, v))) return rc;
        int nl = L.step(v, d->odd, stats, k, d->stats, c->stream, &c->side);
        c->launches += nl - 1;
        if ((rc = launchBox(c))) return rc;
        d->odd = !d->odd;
        d->pending = hasFaces;
        d->steps += 1;
        if (recompute) {   // the streamed state, before the boundary processors
            nl = L.rhoBarJ(d->view(), d->odd, 0, d->bbRho, c->stream);
            c->launches += nl - 1;
            if ((rc = launchBox(c))) return rc;
        }
        if ((rc = finishSurface(c, d))) return rc;
    }
    if (collect_stats) d->statsValid = true;
    return PLBGPU_OK;
}

int plbgpu_time_steps(plbgpu_ctx* c, int h, int nsteps, int collect_stats, float* ms) {
    if (!c || !ms) return PLBGPU_ERR_ARG;
    cudaEvent_t e0, e1;
    CUDA_TRY(c, cudaEventCreate(&e0));
    CUDA_TRY(c, cudaEventCreate(&e1));
    CUDA_TRY(c, cudaEventRecord(e0, c->stream));
    int rc = plbgpu_collide_and_stream(c, h, nsteps, collect_stats);
    if (rc) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rc;
    }
    CUDA_TRY(c, cudaEventRecord(e1, c->stream));
    CUDA_TRY(c, cudaEventSynchronize(e1));
    CUDA_TRY(c, cudaEventElapsedTime(ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    Domain* d;
    if ((rc = lookup(c, h, &d))) return rc;
    return checkStatus(c, d);
}


// ------------------------------------------------------------ binary-block checkpoints

namespace {

// Values per cell of each block kind (sizeOfCell / sizeof(T): the populations
// and the external scalars of the descriptor, or the field's components).
int blockWidth(int what) {
    switch (what) {
    case PLBGPU_BLOCK_LATTICE: return 19;
    case PLBGPU_BLOCK_FORCED_LATTICE: return 22;
    case PLBGPU_BLOCK_DENSITY: return 1;
    case PLBGPU_BLOCK_VELOCITY: return 3;
    case PLBGPU_BLOCK_RHOBAR: return 1;
    case PLBGPU_BLOCK_J: return 3;
    default: return 0;
    }
}

void hostBase64(const unsigned char* in, size_t n, std::string& out) {
    static const char a[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    for (size_t i = 0; i < n; i += 3) {
        unsigned b0 = in[i], b1 = i + 1 < n ? in[i + 1] : 0u, b2 = i + 2 < n ? in[i + 2] : 0u;
        out += a[b0 >> 2];
        out += a[((b0 & 3u) << 4) | (b1 >> 4)];
        out += i + 1 < n ? a[((b1 & 15u) << 2) | (b2 >> 6)] : '=';
        out += i + 2 < n ? a[b2 & 63u] : '=';
    }
}

// Device buffers of one save / load, freed on every exit path.
struct Ckpt {
    double* rec = nullptr;     // records of one slab
    double* tmp = nullptr;     // gathered columns
    uint8_t* bytes = nullptr;  // decoded bytes of one slab (+ the partial quads around it)
    char* text = nullptr;      // base64 of one slab
    uint8_t* head = nullptr;   // up to two bytes carried to the next slab
    unsigned* bad = nullptr;
    ~Ckpt() {
        cudaFree(rec); cudaFree(tmp); cudaFree(bytes); cudaFree(text); cudaFree(head); cudaFree(bad);
    }
};

struct FileCloser {
    FILE* f;
    ~FileCloser() { if (f) fclose(f); }
};

int ckptAlloc(plbgpu_ctx* c, Ckpt& k, long long cells, int w) {
    const size_t recBytes = (size_t)cells * w * sizeof(double);
    CUDA_TRY(c, cudaMalloc(&k.rec, recBytes));
    CUDA_TRY(c, cudaMalloc(&k.tmp, (size_t)cells * 19 * sizeof(double)));
    CUDA_TRY(c, cudaMalloc(&k.bytes, recBytes + 8));
    CUDA_TRY(c, cudaMalloc(&k.text, 4 * ((recBytes + 2) / 3 + 2)));
    CUDA_TRY(c, cudaMalloc(&k.head, 4));
    CUDA_TRY(c, cudaMalloc(&k.bad, sizeof(unsigned)));
    CUDA_TRY(c, cudaMemsetAsync(k.bad, 0, sizeof(unsigned), c->stream));
    return PLBGPU_OK;
}

// Whole x-planes per slab: about 32 MB of records, at least one plane.
int slabPlanes(const Domain* d, int w) {
    long long plane = (long long)d->ny * d->nz * w * (long long)sizeof(double);
    long long p = (32ll << 20) / (plane > 0 ? plane : 1);
    return (int)(p < 1 ? 1 : (p > d->nx ? d->nx : p));
}

// Records of box b (one cell after another, x-major, z fastest) into k.rec.
int buildRecords(plbgpu_ctx* c, Domain* d, int what, const Box& b, Ckpt& k) {
    const Launchers& L = launchers(d->precision);
    const int pending = d->pending && d->bc ? 1 : 0;
    const int w = blockWidth(what);
    const long long cells = boxCells(b);
    int nl = 1, rc;
    if (what == PLBGPU_BLOCK_LATTICE) {
        nl = L.extract(d->view(), d->odd, b, pending, k.rec, c->stream);
    } else if (what == PLBGPU_BLOCK_FORCED_LATTICE) {
        nl = L.extract(d->view(), d->odd, b, pending, k.tmp, c->stream);
        launchColumns(k.tmp, 19, 0, 19, k.rec, 22, 0, cells, c->stream);
        dim3 g = rowGrid(b.z1 - b.z0 + 1, b.y1 - b.y0 + 1, b.x1 - b.x0 + 1, 128);
        if (!d->force)
            CUDA_TRY(c, cudaMemsetAsync(k.tmp, 0, sizeof(double) * 3 * cells, c->stream));
        else if (d->precision == PLBGPU_FP64)
            boxPlanesKernel<double, double><<<g, 128, 0, c->stream>>>(static_cast<double*>(d->force), d->n, d->ny,
                                                                      d->nz, b, k.tmp, 3, 1);
        else
            boxPlanesKernel<float, double><<<g, 128, 0, c->stream>>>(static_cast<float*>(d->force), d->n, d->ny,
                                                                     d->nz, b, k.tmp, 3, 1);
        launchColumns(k.tmp, 3, 0, 3, k.rec, 22, 19, cells, c->stream);
        nl = 4;
    } else if (what == PLBGPU_BLOCK_DENSITY || what == PLBGPU_BLOCK_VELOCITY) {
        nl = L.field(d->view(), d->odd, b, pending, (double)1 / d->rho0, d->bbRho,
                     what == PLBGPU_BLOCK_DENSITY ? 1 : 0, k.rec, c->stream);
    } else {
        if ((rc = extBox(c, d, b, k.tmp, 1))) return rc;
        launchColumns(k.tmp, 4, what == PLBGPU_BLOCK_RHOBAR ? 0 : 1, w, k.rec, w, 0, cells, c->stream);
        nl = 1;
    }
    c->launches += nl - 1;
    return launchBox(c);
}

// The records in k.rec become the contents of box b.
int applyRecords(plbgpu_ctx* c, Domain* d, int what, const Box& b, Ckpt& k) {
    const Launchers& L = launchers(d->precision);
    const int w = blockWidth(what);
    const long long cells = boxCells(b);
    int nl = 1;
    dim3 g = rowGrid(b.z1 - b.z0 + 1, b.y1 - b.y0 + 1, b.x1 - b.x0 + 1, 128);
    if (what == PLBGPU_BLOCK_LATTICE) {
        nl = L.insert(d->view(), d->odd, b, k.rec, c->stream);
    } else if (what == PLBGPU_BLOCK_FORCED_LATTICE) {
        launchColumns(k.rec, 22, 0, 19, k.tmp, 19, 0, cells, c->stream);
        nl = L.insert(d->view(), d->odd, b, k.tmp, c->stream);
        launchColumns(k.rec, 22, 19, 3, k.tmp, 3, 0, cells, c->stream);
        if (d->precision == PLBGPU_FP64)
            boxPlanesKernel<double, double><<<g, 128, 0, c->stream>>>(static_cast<double*>(d->force), d->n, d->ny,
                                                                      d->nz, b, k.tmp, 3, 0);
        else
            boxPlanesKernel<float, double><<<g, 128, 0, c->stream>>>(static_cast<float*>(d->force), d->n, d->ny,
                                                                     d->nz, b, k.tmp, 3, 0);
        nl += 3;
    } else {
        const long long off = what == PLBGPU_BLOCK_RHOBAR ? 0 : d->n;
        if (d->precision == PLBGPU_FP64)
            boxPlanesKernel<double, double><<<g, 128, 0, c->stream>>>(static_cast<double*>(d->ext) + off, d->n, d->ny,
                                                                      d->nz, b, k.rec, w, 0);
        else
            boxPlanesKernel<float, double><<<g, 128, 0, c->stream>>>(static_cast<float*>(d->ext) + off, d->n, d->ny,
                                                                     d->nz, b, k.rec, w, 0);
    }
    c->launches += nl - 1;
    return launchBox(c);
}

// What a load into `what` needs allocated, after the pending faces are done.
int prepareLoad(plbgpu_ctx* c, Domain* d, int what) {
    int rc;
    if ((rc = materialize(c, d))) return rc;
    if (what == PLBGPU_BLOCK_FORCED_LATTICE && (rc = ensureAux(c, d, false, true, false))) return rc;
    if ((what == PLBGPU_BLOCK_RHOBAR || what == PLBGPU_BLOCK_J) && (rc = ensureExt(c, d))) return rc;
    return PLBGPU_OK;
}

}  // namespace

int plbgpu_save_binary_block(plbgpu_ctx* c, int h, int what, const char* path, int enforce_uint) {
    ProfRange prof("io");
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    const int w = blockWidth(what);
    if (!w) return fail(c, PLBGPU_ERR_ARG, "unknown block kind %d", what);
    if (!path) return fail(c, PLBGPU_ERR_ARG, "null path");
    if ((what == PLBGPU_BLOCK_RHOBAR || what == PLBGPU_BLOCK_J) && !d->ext)
        return fail(c, PLBGPU_ERR_STATE, "no rho-bar/j fields to save");
    if ((rc = checkStatus(c, d))) return rc;
    FileCloser fc{fopen(path, "wb")};
    if (!fc.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s for writing", path);
    // Size header, encoded on its own (io/serializerIO.cpp:64-80).
    const unsigned long long size = (unsigned long long)d->n * w * sizeof(double);
    std::string hdr;
    if (enforce_uint) {
        if (size > 0xffffffffull) return fail(c, PLBGPU_ERR_ARG, "%llu bytes do not fit a 32-bit header", size);
        unsigned u = (unsigned)size;
        hostBase64(reinterpret_cast<const unsigned char*>(&u), sizeof(u), hdr);
    } else {
        hostBase64(reinterpret_cast<const unsigned char*>(&size), sizeof(size), hdr);
    }
    if (fwrite(hdr.data(), 1, hdr.size(), fc.f) != hdr.size()) return fail(c, PLBGPU_ERR_ARG, "write to %s failed", path);
    const int planes = slabPlanes(d, w);
    Ckpt k;
    if ((rc = ckptAlloc(c, k, (long long)planes * d->ny * d->nz, w))) return rc;
    std::vector<char> text;
    int headLen = 0;
    for (int x0 = 0; x0 < d->nx; x0 += planes) {
        const int x1 = x0 + planes - 1 < d->nx - 1 ? x0 + planes - 1 : d->nx - 1;
        Box b{x0, x1, 0, d->ny - 1, 0, d->nz - 1};
        const long long cells = boxCells(b);
        if ((rc = buildRecords(c, d, what, b, k))) return rc;
        const size_t bodyLen = (size_t)cells * w * sizeof(double);
        const size_t total = (size_t)headLen + bodyLen;
        const bool last = x1 == d->nx - 1;
        const size_t quads = last ? (total + 2) / 3 : total / 3;
        launchBase64Encode(k.head, headLen, reinterpret_cast<const uint8_t*>(k.rec), bodyLen, quads, k.text,
                           c->stream);
        if ((rc = launchBox(c))) return rc;
        const int carry = last ? 0 : (int)(total - 3 * quads);
        if (carry)
            CUDA_TRY(c, cudaMemcpyAsync(k.head, reinterpret_cast<const uint8_t*>(k.rec) + bodyLen - carry, carry,
                                        cudaMemcpyDeviceToDevice, c->stream));
        headLen = carry;
        text.resize(4 * quads);
        CUDA_TRY(c, cudaMemcpyAsync(text.data(), k.text, text.size(), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        if (fwrite(text.data(), 1, text.size(), fc.f) != text.size())
            return fail(c, PLBGPU_ERR_ARG, "write to %s failed", path);
    }
    if (fflush(fc.f) != 0) return fail(c, PLBGPU_ERR_ARG, "write to %s failed", path);
    return PLBGPU_OK;
}

int plbgpu_load_binary_block(plbgpu_ctx* c, int h, int what, const char* path, int enforce_uint) {
    ProfRange prof("io");
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    const int w = blockWidth(what);
    if (!w) return fail(c, PLBGPU_ERR_ARG, "unknown block kind %d", what);
    if (what == PLBGPU_BLOCK_DENSITY || what == PLBGPU_BLOCK_VELOCITY)
        return fail(c, PLBGPU_ERR_ARG, "density and velocity blocks are derived data and cannot be loaded");
    if (!path) return fail(c, PLBGPU_ERR_ARG, "null path");
    FileCloser fc{fopen(path, "rb")};
    if (!fc.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s", path);
    const long hdrChars = enforce_uint ? 8 : 12;
    char hdr[12];
    if (fread(hdr, 1, hdrChars, fc.f) != (size_t)hdrChars) return fail(c, PLBGPU_ERR_ARG, "%s: short header", path);
    unsigned long long size = 0;
    {
        unsigned char raw[9] = {0};
        for (long q = 0; q < hdrChars / 4; ++q) {
            unsigned v[4];
            for (int i = 0; i < 4; ++i) {
                unsigned char ch = (unsigned char)hdr[4 * q + i];
                v[i] = ch >= 'A' && ch <= 'Z' ? ch - 'A' : ch >= 'a' && ch <= 'z' ? ch - 'a' + 26
                     : ch >= '0' && ch <= '9' ? ch - '0' + 52 : ch == '+' ? 62u : ch == '/' ? 63u : 0u;
            }
            unsigned char b[3] = {(unsigned char)((v[0] << 2) | (v[1] >> 4)),
                                  (unsigned char)(((v[1] & 15u) << 4) | (v[2] >> 2)),
                                  (unsigned char)(((v[2] & 3u) << 6) | v[3])};
            for (int i = 0; i < 3 && 3 * q + i < 9; ++i) raw[3 * q + i] = b[i];
        }
        if (enforce_uint) {
            unsigned u;
            memcpy(&u, raw, 4);
            size = u;
        } else {
            memcpy(&size, raw, 8);
        }
    }
    const unsigned long long want = (unsigned long long)d->n * w * sizeof(double);
    if (size != want)
        return fail(c, PLBGPU_ERR_ARG, "%s holds %llu bytes, the %dx%dx%d domain needs %llu", path, size, d->nx, d->ny,
                    d->nz, want);
    if ((rc = prepareLoad(c, d, what))) return rc;
    const int planes = slabPlanes(d, w);
    Ckpt k;
    if ((rc = ckptAlloc(c, k, (long long)planes * d->ny * d->nz, w))) return rc;
    const unsigned long long totalQuads = (size + 2) / 3;
    std::vector<char> text;
    for (int x0 = 0; x0 < d->nx; x0 += planes) {
        const int x1 = x0 + planes - 1 < d->nx - 1 ? x0 + planes - 1 : d->nx - 1;
        Box b{x0, x1, 0, d->ny - 1, 0, d->nz - 1};
        const long long cells = boxCells(b);
        const unsigned long long start = (unsigned long long)x0 * d->ny * d->nz * w * sizeof(double);
        const unsigned long long end = start + (unsigned long long)cells * w * sizeof(double);
        const unsigned long long q0 = start / 3, q1 = (end + 2) / 3 < totalQuads ? (end + 2) / 3 : totalQuads;
        text.resize(4 * (q1 - q0));
        if (fseek(fc.f, hdrChars + (long)(4 * q0), SEEK_SET) != 0 ||
            fread(text.data(), 1, text.size(), fc.f) != text.size())
            return fail(c, PLBGPU_ERR_ARG, "%s: truncated data", path);
        CUDA_TRY(c, cudaMemcpyAsync(k.text, text.data(), text.size(), cudaMemcpyHostToDevice, c->stream));
        const unsigned long long held = (3 * q1 < size ? 3 * q1 : size) - 3 * q0;
        launchBase64Decode(k.text, q1 - q0, held, k.bytes, k.bad, c->stream);
        if ((rc = launchBox(c))) return rc;
        CUDA_TRY(c, cudaMemcpyAsync(k.rec, k.bytes + (start - 3 * q0), end - start, cudaMemcpyDeviceToDevice,
                                    c->stream));
        unsigned bad = 0;
        CUDA_TRY(c, cudaMemcpyAsync(&bad, k.bad, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        if (bad) return fail(c, PLBGPU_ERR_ARG, "%s: not base64 data", path);
        if ((rc = applyRecords(c, d, what, b, k))) return rc;
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (what == PLBGPU_BLOCK_LATTICE || what == PLBGPU_BLOCK_FORCED_LATTICE) d->statsValid = false;
    return PLBGPU_OK;
}

// ------------------------------------------------------------ parallel-I/O states

namespace {

// Family, descriptor and cell size of a block kind as parallelIO::save
// describes it (io/multiBlockWriter3D.cpp:53-137).
bool isLatticeBlock(int what) { return what == PLBGPU_BLOCK_LATTICE || what == PLBGPU_BLOCK_FORCED_LATTICE; }

void stateTypeInfo(int what, const char** family, const char** descriptor) {
    switch (what) {
    case PLBGPU_BLOCK_LATTICE: *family = "BlockLattice3D"; *descriptor = "D3Q19"; return;
    case PLBGPU_BLOCK_FORCED_LATTICE: *family = "BlockLattice3D"; *descriptor = "ForcedD3Q19"; return;
    case PLBGPU_BLOCK_DENSITY: case PLBGPU_BLOCK_RHOBAR: *family = "ScalarField3D"; *descriptor = nullptr; return;
    default: *family = "TensorField3D"; *descriptor = nullptr; return;
    }
}

// Text of the first <tag ...> ... </tag> element at or after `from` (attributes
// allowed); npos when absent.  `next` receives the position after it.
size_t xmlElement(const std::string& doc, const std::string& tag, size_t from, std::string& text, size_t* next) {
    size_t a = from;
    while ((a = doc.find("<" + tag, a)) != std::string::npos) {
        const char after = a + 1 + tag.size() < doc.size() ? doc[a + 1 + tag.size()] : '\0';
        if (after == '>' || after == ' ') break;
        a += 1;
    }
    if (a == std::string::npos) return a;
    const size_t open = doc.find('>', a);
    const size_t close = doc.find("</" + tag + ">", open);
    if (open == std::string::npos || close == std::string::npos) return std::string::npos;
    text = doc.substr(open + 1, close - open - 1);
    if (next) *next = close + tag.size() + 3;
    return a;
}

bool parseLongs(const std::string& text, std::vector<long long>& out) {
    out.clear();
    const char* p = text.c_str();
    while (*p) {
        while (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r') ++p;
        if (!*p) break;
        char* e = nullptr;
        long long v = strtoll(p, &e, 10);
        if (e == p) return false;
        out.push_back(v);
        p = e;
    }
    return true;
}

// The description <base>.plb of a one-component state, in the layout of the
// reference's XML writer (io/multiBlockWriter3D.cpp:53-137,
// libraryInterfaces/TINYXML_xmlIO.hh:229-272).  dict: the DynamicsDict of a
// state with dynamic content (name -> id, in name order), null for static
// content.
std::string processorList(const Domain* d, const char* descriptor);

std::string stateDescription(const Domain* d, int what, const std::string& datName, unsigned long long bytes,
                             const std::map<std::string, int>* dict) {
    const int w = blockWidth(what);
    const char *family, *descriptor;
    stateTypeInfo(what, &family, &descriptor);
    char buf[512];
    std::string x = "<?xml version=\"1.0\" ?>\n<Block3D>\n    <General>\n";
    x += std::string("        <Family> ") + family + " </Family>\n        <Datatype> double </Datatype>\n";
    if (descriptor) x += std::string("        <Descriptor> ") + descriptor + " </Descriptor>\n";
    snprintf(buf, sizeof(buf),
             "        <cellDim> %d </cellDim>\n        <dynamicContent> %s </dynamicContent>\n"
             "        <globalId> 0 </globalId>\n    </General>\n    <Structure>\n"
             "        <BoundingBox> 0 %d 0 %d 0 %d </BoundingBox>\n        <EnvelopeWidth> 1 </EnvelopeWidth>\n"
             "        <GridLevel> 0 </GridLevel>\n        <NumComponents> 1 </NumComponents>\n    </Structure>\n"
             "    <Data>\n",
             w, dict ? "True" : "False", d->nx - 1, d->ny - 1, d->nz - 1);
    x += buf;
    x += "        <File> " + datName + " </File>\n";
    snprintf(buf, sizeof(buf), "        <Component> 0 %d 0 %d 0 %d </Component>\n        <Offsets> %llu </Offsets>\n",
             d->nx - 1, d->ny - 1, d->nz - 1, bytes);
    x += buf;
    if (dict && !dict->empty()) {
        x += "        <DynamicsDict>\n";
        for (const auto& e : *dict) x += "            <" + e.first + "> " + std::to_string(e.second) + " </" + e.first + ">\n";
        x += "        </DynamicsDict>\n";
    }
    if (isLatticeBlock(what)) x += processorList(d, descriptor);
    x += "    </Data>\n</Block3D>\n";
    return x;
}

// The <Processor> entries of a lattice description, indexed by their place
// in the list (io/multiBlockWriter3D.cpp:113-136), as the reference's XML
// writer prints an indexed element (libraryInterfaces/TINYXML_xmlIO.hh:
// 229-272): the id attribute unless the list is one entry, and each value
// between single spaces.
std::string processorList(const Domain* d, const char* descriptor) {
    // a leaf element: the text between single spaces, nothing when empty
    auto leaf = [](const char* tag, const std::string& text) {
        return std::string("            <") + tag + ">" + (text.empty() ? "" : " " + text + " ") + "</" + tag + ">\n";
    };
    auto joined = [](const long long* v, size_t n) {
        std::string t;
        for (size_t i = 0; i < n; ++i) t += (i ? " " : "") + std::to_string(v[i]);
        return t;
    };
    std::string x;
    const bool ids = d->processors.size() > 1;
    const std::string td = std::string("double_") + descriptor;
    for (size_t i = 0; i < d->processors.size(); ++i) {
        const ProcessorRecord& r = d->processors[i];
        std::string name = r.name;
        for (size_t p; (p = name.find("%TD")) != std::string::npos;) name.replace(p, 3, td);
        x += ids ? "        <Processor id=\"" + std::to_string(i) + "\">\n" : std::string("        <Processor>\n");
        x += leaf("Name", name) + leaf("Domain", joined(r.domain, 6)) + leaf("Data", r.data) +
             leaf("Level", std::to_string(r.level)) + leaf("Blocks", joined(r.blocks.data(), r.blocks.size()));
        x += "        </Processor>\n";
    }
    return x;
}

}  // namespace

int plbgpu_save_state(plbgpu_ctx* c, int h, int what, const char* base) {
    ProfRange prof("io");
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    const int w = blockWidth(what);
    if (!w) return fail(c, PLBGPU_ERR_ARG, "unknown block kind %d", what);
    if (!base) return fail(c, PLBGPU_ERR_ARG, "null path");
    if ((what == PLBGPU_BLOCK_RHOBAR || what == PLBGPU_BLOCK_J) && !d->ext)
        return fail(c, PLBGPU_ERR_STATE, "no rho-bar/j fields to save");
    if ((rc = checkStatus(c, d))) return rc;
    const std::string datName = std::string(base) + ".dat", plbName = std::string(base) + ".plb";
    // Raw records of the one component, the whole bounding box
    // (writeRawData, io/mpiParallelIO.cpp:92-150).
    {
        FileCloser fc{fopen(datName.c_str(), "wb")};
        if (!fc.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s for writing", datName.c_str());
        const int planes = slabPlanes(d, w);
        Ckpt k;
        if ((rc = ckptAlloc(c, k, (long long)planes * d->ny * d->nz, w))) return rc;
        std::vector<char> host;
        for (int x0 = 0; x0 < d->nx; x0 += planes) {
            const int x1 = x0 + planes - 1 < d->nx - 1 ? x0 + planes - 1 : d->nx - 1;
            Box b{x0, x1, 0, d->ny - 1, 0, d->nz - 1};
            if ((rc = buildRecords(c, d, what, b, k))) return rc;
            host.resize((size_t)boxCells(b) * w * sizeof(double));
            CUDA_TRY(c, cudaMemcpyAsync(host.data(), k.rec, host.size(), cudaMemcpyDeviceToHost, c->stream));
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            if (fwrite(host.data(), 1, host.size(), fc.f) != host.size())
                return fail(c, PLBGPU_ERR_ARG, "write to %s failed", datName.c_str());
        }
        if (fflush(fc.f) != 0) return fail(c, PLBGPU_ERR_ARG, "write to %s failed", datName.c_str());
    }
    const std::string x = stateDescription(d, what, datName, (unsigned long long)d->n * w * sizeof(double), nullptr);
    FileCloser fp{fopen(plbName.c_str(), "wb")};
    if (!fp.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s for writing", plbName.c_str());
    if (fwrite(x.data(), 1, x.size(), fp.f) != x.size() || fflush(fp.f) != 0)
        return fail(c, PLBGPU_ERR_ARG, "write to %s failed", plbName.c_str());
    return PLBGPU_OK;
}

namespace {

// What <base>.plb says (readXmlSpec, io/multiBlockReader3D.cpp:135-212, and
// createDynamicsForeignIds3D, :67-90); component boxes relative to the
// bounding box, whose size must be the domain's.
struct StateSpec {
    bool dynamic = false;
    std::vector<Box> comps;
    std::vector<long long> offsets;
    std::string datName;
    std::map<int, std::string> names;   // DynamicsDict: id -> dynamics name
};

int parseStateSpec(plbgpu_ctx* c, const Domain* d, const char* plb, int w, StateSpec& s) {
    std::string doc;
    {
        FileCloser fc{fopen(plb, "rb")};
        if (!fc.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s", plb);
        char chunk[4096];
        size_t got;
        while ((got = fread(chunk, 1, sizeof(chunk), fc.f)) > 0) doc.append(chunk, got);
    }
    std::string t;
    std::vector<long long> v;
    if (xmlElement(doc, "cellDim", 0, t, nullptr) == std::string::npos || !parseLongs(t, v) || v.size() != 1)
        return fail(c, PLBGPU_ERR_ARG, "%s: no cellDim", plb);
    if (v[0] != w) return fail(c, PLBGPU_ERR_ARG, "%s: cells of %lld values, this block kind has %d", plb, v[0], w);
    if (xmlElement(doc, "dynamicContent", 0, t, nullptr) == std::string::npos)
        return fail(c, PLBGPU_ERR_ARG, "%s: no dynamicContent", plb);
    s.dynamic = t.find("True") != std::string::npos;
    std::vector<long long> bb;
    if (xmlElement(doc, "BoundingBox", 0, t, nullptr) == std::string::npos || !parseLongs(t, bb) || bb.size() != 6)
        return fail(c, PLBGPU_ERR_ARG, "%s: no bounding box", plb);
    if (bb[1] - bb[0] + 1 != d->nx || bb[3] - bb[2] + 1 != d->ny || bb[5] - bb[4] + 1 != d->nz)
        return fail(c, PLBGPU_ERR_ARG, "%s: a %lldx%lldx%lld block, the domain is %dx%dx%d", plb, bb[1] - bb[0] + 1,
                    bb[3] - bb[2] + 1, bb[5] - bb[4] + 1, d->nx, d->ny, d->nz);
    if (xmlElement(doc, "Offsets", 0, t, nullptr) == std::string::npos || !parseLongs(t, s.offsets))
        return fail(c, PLBGPU_ERR_ARG, "%s: no offsets", plb);
    std::string datName;
    if (xmlElement(doc, "File", 0, datName, nullptr) == std::string::npos)
        return fail(c, PLBGPU_ERR_ARG, "%s: no data file", plb);
    const size_t s0 = datName.find_first_not_of(" \n\t\r"), s1 = datName.find_last_not_of(" \n\t\r");
    datName = s0 == std::string::npos ? std::string() : datName.substr(s0, s1 - s0 + 1);
    if (datName.find('/') == std::string::npos) {   // next to the description
        const std::string p(plb);
        const size_t slash = p.rfind('/');
        if (slash != std::string::npos) datName = p.substr(0, slash + 1) + datName;
    }
    if (datName.size() < 4 || datName.compare(datName.size() - 4, 4, ".dat") != 0) datName += ".dat";
    s.datName = datName;
    size_t pos = 0, next = 0;
    while (xmlElement(doc, "Component", pos, t, &next) != std::string::npos) {
        if (!parseLongs(t, v) || v.size() != 6) return fail(c, PLBGPU_ERR_ARG, "%s: bad component", plb);
        Box b{(int)(v[0] - bb[0]), (int)(v[1] - bb[0]), (int)(v[2] - bb[2]), (int)(v[3] - bb[2]),
              (int)(v[4] - bb[4]), (int)(v[5] - bb[4])};
        if (b.x0 < 0 || b.y0 < 0 || b.z0 < 0 || b.x1 >= d->nx || b.y1 >= d->ny || b.z1 >= d->nz || b.x0 > b.x1 ||
            b.y0 > b.y1 || b.z0 > b.z1)
            return fail(c, PLBGPU_ERR_ARG, "%s: component outside the bounding box", plb);
        s.comps.push_back(b);
        pos = next;
    }
    if (s.comps.size() != s.offsets.size() || s.comps.empty())
        return fail(c, PLBGPU_ERR_ARG, "%s: %zu components, %zu offsets", plb, s.comps.size(), s.offsets.size());
    // <DynamicsDict> <name> id </name> ... </DynamicsDict>
    if (xmlElement(doc, "DynamicsDict", 0, t, nullptr) != std::string::npos) {
        size_t p = 0;
        while ((p = t.find('<', p)) != std::string::npos) {
            const size_t gt = t.find('>', p);
            if (gt == std::string::npos) return fail(c, PLBGPU_ERR_ARG, "%s: bad DynamicsDict", plb);
            const std::string name = t.substr(p + 1, gt - p - 1);
            const size_t close = t.find("</" + name + ">", gt);
            if (close == std::string::npos || !parseLongs(t.substr(gt + 1, close - gt - 1), v) || v.size() != 1)
                return fail(c, PLBGPU_ERR_ARG, "%s: bad DynamicsDict entry %s", plb, name.c_str());
            s.names[(int)v[0]] = name;
            p = close + name.size() + 3;
        }
    }
    return PLBGPU_OK;
}

// The cells of a lattice state with dynamic content: per component, its cells
// x-major, each one's dynamics chain then its w static values
// (blockLattice3D.hh:703-722).  recs receives each component's static values
// (x-major over its box, w per cell); cells, when given, each covered cell's
// dynamics (domain-indexed) and seen which cells the components cover.
int readDynamicCells(plbgpu_ctx* c, const Domain* d, const StateSpec& s, int w,
                     std::vector<std::vector<double>>& recs, std::vector<plbgpu_dyn::Cell>* cells,
                     std::vector<uint8_t>* seen) {
    FileCloser fd{fopen(s.datName.c_str(), "rb")};
    if (!fd.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s", s.datName.c_str());
    recs.assign(s.comps.size(), std::vector<double>());
    if (cells) cells->assign((size_t)d->n, plbgpu_dyn::Cell());
    if (seen) seen->assign((size_t)d->n, 0);
    std::vector<char> buf;
    long long begin = 0;
    for (size_t i = 0; i < s.comps.size(); ++i) {
        const Box& cb = s.comps[i];
        if (s.offsets[i] < begin) return fail(c, PLBGPU_ERR_ARG, "%s: offsets out of order", s.datName.c_str());
        buf.resize((size_t)(s.offsets[i] - begin));
        if (fseek(fd.f, (long)begin, SEEK_SET) != 0 || fread(buf.data(), 1, buf.size(), fd.f) != buf.size())
            return fail(c, PLBGPU_ERR_ARG, "%s: truncated data", s.datName.c_str());
        std::vector<double>& rec = recs[i];
        rec.resize((size_t)boxCells(cb) * w);
        size_t pos = 0, j = 0;
        for (int x = cb.x0; x <= cb.x1; ++x)
            for (int y = cb.y0; y <= cb.y1; ++y)
                for (int z = cb.z0; z <= cb.z1; ++z, ++j) {
                    const size_t idx = ((size_t)x * d->ny + y) * d->nz + z;
                    plbgpu_dyn::Cell cell;
                    const std::string err =
                        plbgpu_dyn::readCell(buf.data(), buf.size(), pos, s.names, x, y, z, d->nx, d->ny, d->nz, cell);
                    if (!err.empty())
                        return fail(c, PLBGPU_ERR_ARG, "%s: cell (%d, %d, %d): %s", s.datName.c_str(), x, y, z,
                                    err.c_str());
                    if (pos + w * sizeof(double) > buf.size())
                        return fail(c, PLBGPU_ERR_ARG, "%s: truncated data", s.datName.c_str());
                    memcpy(&rec[j * w], buf.data() + pos, w * sizeof(double));
                    pos += w * sizeof(double);
                    if (seen) (*seen)[idx] = 1;
                    if (cells) (*cells)[idx] = cell;
                }
        if (pos != buf.size())
            return fail(c, PLBGPU_ERR_ARG, "%s: component %zu has %zu bytes beyond its cells", s.datName.c_str(), i,
                        buf.size() - pos);
        begin = s.offsets[i];
    }
    return PLBGPU_OK;
}

// Host records of box cb (x-major, blockWidth(what) per cell) into the domain,
// slab by slab.
int uploadRecords(plbgpu_ctx* c, Domain* d, int what, const Box& cb, const std::vector<double>& rec) {
    const int w = blockWidth(what);
    const long long plane = (long long)(cb.y1 - cb.y0 + 1) * (cb.z1 - cb.z0 + 1);
    long long per = (32ll << 20) / (plane * w * (long long)sizeof(double));
    const int planes = (int)(per < 1 ? 1 : (per > cb.x1 - cb.x0 + 1 ? cb.x1 - cb.x0 + 1 : per));
    Ckpt k;
    int rc;
    if ((rc = ckptAlloc(c, k, (long long)planes * plane, w))) return rc;
    for (int x0 = cb.x0; x0 <= cb.x1; x0 += planes) {
        const int x1 = x0 + planes - 1 < cb.x1 ? x0 + planes - 1 : cb.x1;
        Box b{x0, x1, cb.y0, cb.y1, cb.z0, cb.z1};
        const size_t first = (size_t)(x0 - cb.x0) * plane * w;
        CUDA_TRY(c, cudaMemcpyAsync(k.rec, rec.data() + first, (size_t)boxCells(b) * w * sizeof(double),
                                    cudaMemcpyHostToDevice, c->stream));
        if ((rc = applyRecords(c, d, what, b, k))) return rc;
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    }
    return PLBGPU_OK;
}


}  // namespace

int plbgpu_load_state(plbgpu_ctx* c, int h, int what, const char* plb) {
    ProfRange prof("io");
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    const int w = blockWidth(what);
    if (!w) return fail(c, PLBGPU_ERR_ARG, "unknown block kind %d", what);
    if (what == PLBGPU_BLOCK_DENSITY || what == PLBGPU_BLOCK_VELOCITY)
        return fail(c, PLBGPU_ERR_ARG, "density and velocity blocks are derived data and cannot be loaded");
    if (!plb) return fail(c, PLBGPU_ERR_ARG, "null path");
    StateSpec s;
    if ((rc = parseStateSpec(c, d, plb, w, s))) return rc;
    if (s.dynamic && isLatticeBlock(what)) {
        // load(plb, lattice, false) of a state with dynamic content: the
        // populations (and force) only, the dynamics chains are skipped.
        std::vector<std::vector<double>> recs;
        if ((rc = readDynamicCells(c, d, s, w, recs, nullptr, nullptr))) return rc;
        if ((rc = prepareLoad(c, d, what))) return rc;
        for (size_t i = 0; i < s.comps.size(); ++i)
            if ((rc = uploadRecords(c, d, what, s.comps[i], recs[i]))) return rc;
        d->statsValid = false;
        return PLBGPU_OK;
    }
    // Static content (a field's records are the same with or without it:
    // ScalarFieldDataTransfer3D ignores the kind, dataField3D.hh:133-150).
    FileCloser fd{fopen(s.datName.c_str(), "rb")};
    if (!fd.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s", s.datName.c_str());
    if ((rc = prepareLoad(c, d, what))) return rc;
    std::vector<char> host;
    long long begin = 0;
    for (size_t i = 0; i < s.comps.size(); ++i) {
        const Box& cb = s.comps[i];
        const long long bytes = s.offsets[i] - begin;
        if (bytes != boxCells(cb) * w * (long long)sizeof(double))
            return fail(c, PLBGPU_ERR_ARG, "%s: component %zu holds %lld bytes, its box needs %lld", plb, i, bytes,
                        boxCells(cb) * w * (long long)sizeof(double));
        if (fseek(fd.f, (long)begin, SEEK_SET) != 0) return fail(c, PLBGPU_ERR_ARG, "%s: truncated", s.datName.c_str());
        // whole x-planes of the component at a time
        const long long plane = (long long)(cb.y1 - cb.y0 + 1) * (cb.z1 - cb.z0 + 1) * w * sizeof(double);
        long long per = (32ll << 20) / (plane > 0 ? plane : 1);
        const int planes = (int)(per < 1 ? 1 : (per > cb.x1 - cb.x0 + 1 ? cb.x1 - cb.x0 + 1 : per));
        Ckpt k;
        if ((rc = ckptAlloc(c, k, (long long)planes * (cb.y1 - cb.y0 + 1) * (cb.z1 - cb.z0 + 1), w))) return rc;
        for (int x0 = cb.x0; x0 <= cb.x1; x0 += planes) {
            const int x1 = x0 + planes - 1 < cb.x1 ? x0 + planes - 1 : cb.x1;
            Box b{x0, x1, cb.y0, cb.y1, cb.z0, cb.z1};
            host.resize((size_t)boxCells(b) * w * sizeof(double));
            if (fread(host.data(), 1, host.size(), fd.f) != host.size())
                return fail(c, PLBGPU_ERR_ARG, "%s: truncated data", s.datName.c_str());
            CUDA_TRY(c, cudaMemcpyAsync(k.rec, host.data(), host.size(), cudaMemcpyHostToDevice, c->stream));
            if ((rc = applyRecords(c, d, what, b, k))) return rc;
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        }
        begin = s.offsets[i];
    }
    if (isLatticeBlock(what)) d->statsValid = false;
    return PLBGPU_OK;
}

int plbgpu_save_state_dynamic(plbgpu_ctx* c, int h, int what, const char* base) {
    ProfRange prof("io");
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (!isLatticeBlock(what)) return fail(c, PLBGPU_ERR_ARG, "dynamic content: block kind %d is not a lattice", what);
    if (!base) return fail(c, PLBGPU_ERR_ARG, "null path");
    if ((rc = checkStatus(c, d))) return rc;
    const int w = blockWidth(what);
    const size_t n = (size_t)d->n;
    // Cell kinds, boundary values and momentum-exchange directions, host side.
    std::vector<uint8_t> kinds(n);
    std::vector<double> bc(d->bc ? 3 * n : 0);
    std::vector<uint32_t> mask(d->mebb ? n : 0);
    CUDA_TRY(c, cudaMemcpyAsync(kinds.data(), d->flags, n, cudaMemcpyDeviceToHost, c->stream));
    if (d->bc) CUDA_TRY(c, cudaMemcpyAsync(bc.data(), d->bc, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (d->mebb)
        CUDA_TRY(c, cudaMemcpyAsync(mask.data(), d->mebb, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    std::map<std::string, int> dict;   // uniqueDynamicsIds over the chains (metaStuffWrapper3D.hh:167-179)
    {
        bool present[K_NKINDS] = {false};
        for (size_t i = 0; i < n; ++i)
            present[kinds[i] < K_NKINDS ? kinds[i] : K_NODYN] = true;   // outside the lattice: NoDynamics
        for (int k = 0; k < K_NKINDS; ++k)
            if (present[k]) {
                dict[plbgpu_dyn::kindName(k)] = plbgpu_dyn::kindId(k);
                if (plbgpu_dyn::isComposite(k)) dict["BGK"] = plbgpu_dyn::kBgkId;
            }
    }
    plbgpu_dyn::Params p;
    p.omega = d->omega;
    p.rho0 = d->rho0;
    p.bbRho = d->bbRho;
    const std::string datName = std::string(base) + ".dat", plbName = std::string(base) + ".plb";
    unsigned long long total = 0;
    {
        FileCloser fc{fopen(datName.c_str(), "wb")};
        if (!fc.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s for writing", datName.c_str());
        const int planes = slabPlanes(d, w);
        Ckpt k;
        if ((rc = ckptAlloc(c, k, (long long)planes * d->ny * d->nz, w))) return rc;
        std::vector<double> host;
        std::vector<char> out;
        for (int x0 = 0; x0 < d->nx; x0 += planes) {
            const int x1 = x0 + planes - 1 < d->nx - 1 ? x0 + planes - 1 : d->nx - 1;
            Box b{x0, x1, 0, d->ny - 1, 0, d->nz - 1};
            if ((rc = buildRecords(c, d, what, b, k))) return rc;
            const size_t cells = (size_t)boxCells(b);
            host.resize(cells * w);
            CUDA_TRY(c, cudaMemcpyAsync(host.data(), k.rec, host.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                        c->stream));
            CUDA_TRY(c, cudaStreamSynchronize(c->stream));
            out.clear();
            const size_t first = (size_t)x0 * d->ny * d->nz;
            for (size_t j = 0; j < cells; ++j) {
                const size_t idx = first + j;
                const double v[3] = {bc.empty() ? 0. : bc[idx], bc.empty() ? 0. : bc[n + idx],
                                     bc.empty() ? 0. : bc[2 * n + idx]};
                plbgpu_dyn::appendCell(out, kinds[idx], v, mask.empty() ? 0u : mask[idx], p);
                const size_t at = out.size();
                out.resize(at + w * sizeof(double));
                memcpy(&out[at], &host[j * w], w * sizeof(double));
            }
            if (fwrite(out.data(), 1, out.size(), fc.f) != out.size())
                return fail(c, PLBGPU_ERR_ARG, "write to %s failed", datName.c_str());
            total += out.size();
        }
        if (fflush(fc.f) != 0) return fail(c, PLBGPU_ERR_ARG, "write to %s failed", datName.c_str());
    }
    const std::string x = stateDescription(d, what, datName, total, &dict);
    FileCloser fp{fopen(plbName.c_str(), "wb")};
    if (!fp.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s for writing", plbName.c_str());
    if (fwrite(x.data(), 1, x.size(), fp.f) != x.size() || fflush(fp.f) != 0)
        return fail(c, PLBGPU_ERR_ARG, "write to %s failed", plbName.c_str());
    return PLBGPU_OK;
}

int plbgpu_load_processors(plbgpu_ctx* c, int h, const char* plb) {
    ProfRange prof("io");
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (!plb) return fail(c, PLBGPU_ERR_ARG, "null path");
    std::string doc;
    {
        FileCloser fc{fopen(plb, "rb")};
        if (!fc.f) return fail(c, PLBGPU_ERR_ARG, "cannot open %s", plb);
        char chunk[4096];
        size_t got;
        while ((got = fread(chunk, 1, sizeof(chunk), fc.f)) > 0) doc.append(chunk, got);
    }
    auto trim = [](const std::string& t) {
        const size_t a = t.find_first_not_of(" \n\t\r"), b = t.find_last_not_of(" \n\t\r");
        return a == std::string::npos ? std::string() : t.substr(a, b - a + 1);
    };
    std::string t;
    std::vector<long long> bb, v;
    if (xmlElement(doc, "BoundingBox", 0, t, nullptr) == std::string::npos || !parseLongs(t, bb) || bb.size() != 6)
        return fail(c, PLBGPU_ERR_ARG, "%s: no bounding box", plb);
    std::string descriptor;
    if (xmlElement(doc, "Descriptor", 0, t, nullptr) != std::string::npos) descriptor = trim(t);
    const std::string td = "double_" + descriptor;
    std::vector<ProcessorRecord> add;
    size_t pos = 0, next = 0;
    while (xmlElement(doc, "Processor", pos, t, &next) != std::string::npos) {
        pos = next;
        ProcessorRecord r;
        std::string f;
        if (xmlElement(t, "Name", 0, f, nullptr) == std::string::npos || trim(f).empty())
            return fail(c, PLBGPU_ERR_ARG, "%s: processor without a name", plb);
        r.name = trim(f);
        if (!descriptor.empty())
            for (size_t p = 0; (p = r.name.find(td, p)) != std::string::npos;) {
                const size_t e = p + td.size();
                if (p > 0 && r.name[p - 1] == '_' && (e == r.name.size() || r.name[e] == '_')) {
                    r.name.replace(p, td.size(), "%TD");
                    p += 3;
                } else {
                    p = e;
                }
            }
        // the writer puts one space on either side of a non-empty text
        if (xmlElement(t, "Data", 0, f, nullptr) == std::string::npos)
            return fail(c, PLBGPU_ERR_ARG, "%s: processor %s without data", plb, r.name.c_str());
        r.data = f.size() >= 2 && f.front() == ' ' && f.back() == ' ' ? f.substr(1, f.size() - 2) : f;
        if (xmlElement(t, "Domain", 0, f, nullptr) == std::string::npos || !parseLongs(f, v) || v.size() != 6)
            return fail(c, PLBGPU_ERR_ARG, "%s: processor %s without a domain", plb, r.name.c_str());
        // readXmlProcessors keeps the processors that meet the block, clipped
        // to it (io/multiBlockReader3D.cpp:91-133); coordinates relative to
        // the bounding box, whose origin is the domain's
        const int ext[3] = {d->nx, d->ny, d->nz};
        bool meets = true;
        for (int a = 0; a < 3; ++a) {
            long long l = v[2 * a] - bb[2 * a], u = v[2 * a + 1] - bb[2 * a];
            l = l < 0 ? 0 : l;
            u = u > ext[a] - 1 ? ext[a] - 1 : u;
            meets = meets && l <= u;
            r.domain[2 * a] = l;
            r.domain[2 * a + 1] = u;
        }
        if (xmlElement(t, "Level", 0, f, nullptr) == std::string::npos || !parseLongs(f, v) || v.size() != 1)
            return fail(c, PLBGPU_ERR_ARG, "%s: processor %s without a level", plb, r.name.c_str());
        r.level = v[0];
        if (xmlElement(t, "Blocks", 0, f, nullptr) == std::string::npos || !parseLongs(f, r.blocks))
            return fail(c, PLBGPU_ERR_ARG, "%s: processor %s without blocks", plb, r.name.c_str());
        if (meets) add.push_back(r);
    }
    d->processors.insert(d->processors.end(), add.begin(), add.end());
    return PLBGPU_OK;
}

int plbgpu_load_state_dynamic(plbgpu_ctx* c, int h, int what, const char* plb) {
    ProfRange prof("io");
    Domain* d;
    int rc = lookup(c, h, &d);
    if (rc) return rc;
    if (!isLatticeBlock(what)) return fail(c, PLBGPU_ERR_ARG, "dynamic content: block kind %d is not a lattice", what);
    if (!plb) return fail(c, PLBGPU_ERR_ARG, "null path");
    const int w = blockWidth(what);
    StateSpec s;
    if ((rc = parseStateSpec(c, d, plb, w, s))) return rc;
    if (!s.dynamic) return fail(c, PLBGPU_ERR_ARG, "%s: the state has no dynamic content", plb);
    std::vector<std::vector<double>> recs;
    std::vector<plbgpu_dyn::Cell> cells;
    std::vector<uint8_t> seen;
    if ((rc = readDynamicCells(c, d, s, w, recs, &cells, &seen))) return rc;
    // Cells outside the lattice of a sparse domain stay outside (the
    // reference copies a loaded state into the blocks that exist); every
    // other cell must be in the state.
    const size_t n = cells.size();
    std::vector<uint8_t> kinds(n);
    CUDA_TRY(c, cudaMemcpyAsync(kinds.data(), d->flags, n, cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    // The GPU lattice holds one omega, one rho0 and one wall density.
    bool haveOmega = false, haveInv = false, haveRho = false, composite = false, mebb = false;
    double omega = d->omega, invRho0 = 0, rho = d->bbRho;
    for (size_t i = 0; i < n; ++i) {
        if (kinds[i] == K_NONE) continue;
        if (!seen[i])
            return fail(c, PLBGPU_ERR_ARG, "%s: the components do not cover the lattice (cell %zu)", plb, i);
        const plbgpu_dyn::Cell& cl = cells[i];
        kinds[i] = (uint8_t)cl.kind;
        composite |= plbgpu_dyn::isComposite(cl.kind);
        mebb |= cl.kind == PLBGPU_MOMENTUM_EXCHANGE;
        if (cl.hasOmega) {
            if (haveOmega && cl.omega != omega) return fail(c, PLBGPU_ERR_ARG, "%s: cells with different omega", plb);
            omega = cl.omega;
            haveOmega = true;
        }
        if (cl.hasInvRho0) {
            if (haveInv && cl.invRho0 != invRho0) return fail(c, PLBGPU_ERR_ARG, "%s: cells with different rho0", plb);
            invRho0 = cl.invRho0;
            haveInv = true;
        }
        if (cl.hasRho) {
            if (haveRho && cl.rho != rho)
                return fail(c, PLBGPU_ERR_ARG, "%s: wall cells (bounce-back, no-dynamics) with different densities",
                            plb);
            rho = cl.rho;
            haveRho = true;
        }
    }
    double rho0 = d->rho0;
    if (haveInv && !plbgpu_dyn::rho0FromInverse(invRho0, rho0))
        return fail(c, PLBGPU_ERR_ARG, "%s: no rho0 has the stored 1/rho0 as its reciprocal", plb);
    if ((rc = plbgpu_set_params(c, h, omega, rho0, rho))) return rc;
    if ((rc = plbgpu_set_kinds(c, h, 0, d->nx - 1, 0, d->ny - 1, 0, d->nz - 1, kinds.data(), n))) return rc;
    if (composite) {
        std::vector<double> bc(3 * n);
        for (size_t i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) bc[a * n + i] = cells[i].bc[a];
        if ((rc = ensureAux(c, d, true, false, false))) return rc;
        CUDA_TRY(c, cudaMemcpyAsync(d->bc, bc.data(), 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    }
    if (mebb) {
        std::vector<uint32_t> mask(n);
        for (size_t i = 0; i < n; ++i) mask[i] = cells[i].mask;
        if ((rc = ensureAux(c, d, false, false, true))) return rc;
        CUDA_TRY(c, cudaMemcpyAsync(d->mebb, mask.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    }
    if ((rc = prepareLoad(c, d, what))) return rc;
    for (size_t i = 0; i < s.comps.size(); ++i)
        if ((rc = uploadRecords(c, d, what, s.comps[i], recs[i]))) return rc;
    d->statsValid = false;
    return PLBGPU_OK;
}

// ------------------------------------------------------------ co-processor form

int plbgpu_cp_add_domain(plbgpu_ctx* c, long nx, long ny, long nz, double omega, int* handle) {
    if (!c || !handle || nx < 1 || ny < 1 || nz < 1 || nx > (1 << 30) || ny > (1 << 30) || nz > (1 << 30)) return 0;
    int h;
    if (plbgpu_add_domain(c, (int)nx, (int)ny, (int)nz, PLBGPU_FP64, &h) != PLBGPU_OK) return 0;
    if (plbgpu_set_params(c, h, omega, 1.0, 0.0) != PLBGPU_OK) return 0;
    *handle = h;
    return 1;
}

int plbgpu_cp_send(plbgpu_ctx* c, int handle, long x0, long x1, long y0, long y1, long z0, long z1, const char* data,
                   size_t nbytes) {
    if (nbytes % (19 * sizeof(double))) {
        fail(c, PLBGPU_ERR_ARG, "co-processor send: %zu bytes is not a whole number of D3Q19 cells", nbytes);
        return 0;
    }
    return plbgpu_send(c, handle, (int)x0, (int)x1, (int)y0, (int)y1, (int)z0, (int)z1,
                       reinterpret_cast<const double*>(data), nbytes / sizeof(double)) == PLBGPU_OK;
}

int plbgpu_cp_receive(plbgpu_ctx* c, int handle, long x0, long x1, long y0, long y1, long z0, long z1, char* data,
                      size_t nbytes) {
    if (nbytes % (19 * sizeof(double))) {
        fail(c, PLBGPU_ERR_ARG, "co-processor receive: %zu bytes is not a whole number of D3Q19 cells", nbytes);
        return 0;
    }
    return plbgpu_receive(c, handle, (int)x0, (int)x1, (int)y0, (int)y1, (int)z0, (int)z1,
                          reinterpret_cast<double*>(data), nbytes / sizeof(double)) == PLBGPU_OK;
}

int plbgpu_cp_add_domain_f32(plbgpu_ctx* c, long nx, long ny, long nz, double omega, int* handle) {
    if (!c || !handle || nx < 1 || ny < 1 || nz < 1 || nx > (1 << 30) || ny > (1 << 30) || nz > (1 << 30)) return 0;
    int h;
    if (plbgpu_add_domain(c, (int)nx, (int)ny, (int)nz, PLBGPU_FP32, &h) != PLBGPU_OK) return 0;
    if (plbgpu_set_params(c, h, omega, 1.0, 0.0) != PLBGPU_OK) return 0;
    *handle = h;
    return 1;
}

int plbgpu_cp_send_f32(plbgpu_ctx* c, int handle, long x0, long x1, long y0, long y1, long z0, long z1,
                       const char* data, size_t nbytes) {
    if (nbytes % (19 * sizeof(float))) {
        fail(c, PLBGPU_ERR_ARG, "co-processor send: %zu bytes is not a whole number of D3Q19 cells", nbytes);
        return 0;
    }
    return plbgpu_send_f32(c, handle, (int)x0, (int)x1, (int)y0, (int)y1, (int)z0, (int)z1,
                           reinterpret_cast<const float*>(data), nbytes / sizeof(float)) == PLBGPU_OK;
}

int plbgpu_cp_receive_f32(plbgpu_ctx* c, int handle, long x0, long x1, long y0, long y1, long z0, long z1,
                          char* data, size_t nbytes) {
    if (nbytes % (19 * sizeof(float))) {
        fail(c, PLBGPU_ERR_ARG, "co-processor receive: %zu bytes is not a whole number of D3Q19 cells", nbytes);
        return 0;
    }
    return plbgpu_receive_f32(c, handle, (int)x0, (int)x1, (int)y0, (int)y1, (int)z0, (int)z1,
                              reinterpret_cast<float*>(data), nbytes / sizeof(float)) == PLBGPU_OK;
}

int plbgpu_cp_collide_and_stream(plbgpu_ctx* c, int handle) {
    // Blocking, as the interface requires (coProcessor3D.h:107-115).
    if (plbgpu_collide_and_stream(c, handle, 1, 0) != PLBGPU_OK) return 0;
    return plbgpu_synchronize(c) == PLBGPU_OK;
}

}  // extern "C"
