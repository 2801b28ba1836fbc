// Time-step launchers of one storage type and AA parity: the row kernel of
// the interior rows, and the edge-row kernel beside it.  Included only by the
// step_<type>_<parity>.cu translation units, each of which instantiates
// stepParity<S, ODD> once.
#pragma once

#include "launchers.cuh"
#include "vecrow.cuh"

namespace plbgpu {

template <typename S>
struct StepLaunch {
    using R = typename StoreT<S>::R;
    static constexpr int kBlock = 128;

    // Row kernel of this storage type: the paired kernel for the 2-byte forms
    // when rows have an even length, the one-cell register kernel otherwise.
    // Two cells per thread: the fastest form of the 2-byte storage types on
    // GB300 (rows of even length).
    static bool pairedRows(const DevLattice& L) { return sizeof(S) == 2 && L.nz % 2 == 0 && L.rowForm != 1; }
    // Eight, four or two cells per thread with packed 128-, 64- or 32-bit
    // population words (vecrow.cuh), on request: bit-identical.  Eight and
    // four cells are 34-43% slower than the paired kernel on GB300 (the packed
    // state of eight cells holds 168 registers, 12 resident warps per SM, too
    // few to keep HBM busy).
    static int vectorCells(const DevLattice& L) {
        if (sizeof(S) != 2) return 0;
        if (L.rowForm == 4 && L.nz % 8 == 0) return 8;
        if (L.rowForm == 2 && L.nz % 8 == 0) return 4;
        if (L.rowForm == 3 && L.nz % 2 == 0) return 2;
        return 0;
    }

    template <bool ODD, bool STATS, bool EXT>
    // slab: the interior rows of L's x-range only (xRow0, xRows), on s alone;
    // the caller steps the slab's border rows
    static int stepSplit(const DevLattice& L, const StepParams<R>& p, StatsAcc* acc, cudaStream_t s,
                         const SideStream* side, bool slab = false) {
        int launched = 0;
        // A sparse domain with tile lists runs its dense tiles (no cell outside
        // the lattice in the 3x3 rows around them, one cell beyond each end)
        // through the interior-row kernels, one block per tile, and its other
        // live tiles through the general addressing, which checks each
        // neighbour's kind; without lists every row goes the general way.
        const bool lists = L.sparse && (L.denseTiles || L.generalTiles || L.maskedTiles);
        const bool general = (L.sparse && !lists) || L.nx < 3 || L.ny < 3;
        const int edgeRows = lists ? L.nGeneral : general ? L.nx * L.ny : 2 * L.ny + 2 * (L.nx - 2);
        const long long interiorRows = lists ? L.nDense : (long long)L.xRows * (L.ny - 2);
        // grid over the interior rows: (blocksPerRow, ny-2, nx-2), the row
        // being (blockIdx.z + 1, blockIdx.y + 1); or one block per dense tile,
        // entry blockIdx.y + gridDim.y * blockIdx.z of the list
        // tilesPerBlock: the tiles one block of the list steps
        auto interiorGrid = [&](int blocksPerRow, int tilesPerBlock) {
            if (!lists) return dim3((unsigned)blocksPerRow, (unsigned)(L.ny - 2), (unsigned)L.xRows);
            const int blocks = (L.nDense + tilesPerBlock - 1) / tilesPerBlock;
            const unsigned gy = (unsigned)(blocks < 65535 ? blocks : 65535);
            return dim3(1u, gy, (unsigned)((blocks + gy - 1) / gy));
        };
        // The border rows run on the side stream (the context's highest
        // priority), beside the interior kernel.  Submission order decides
        // whose blocks take the SMs first: the 2-byte forms submit the
        // interior kernel first and the border blocks take the first slots
        // that free up (2-4% faster); FP32 submits the border kernel first
        // (2% faster); FP64 is bound by its FP64 pipe either way.
        constexpr bool interiorFirst = sizeof(S) == 2;
        cudaStream_t es = s;
        if (side && !general && !slab && cudaEventRecord(side->fork, s) == cudaSuccess &&
            cudaStreamWaitEvent(side->stream, side->fork, 0) == cudaSuccess)
            es = side->stream;
        auto interior = [&]() {
            if (general || interiorRows == 0) return;
            if (const int cpt = vectorCells(L)) {
                if constexpr (sizeof(S) == 2) {
                    Planes<S> pl;
                    RowDeltas d;
                    for (int i = 0; i < 19; ++i) {
                        pl.p[i] = static_cast<S*>(L.pop) + (long long)i * L.stride;
                        d.d[i] = cdir(i, 0) * L.ny * L.nz + cdir(i, 1) * L.nz;
                    }
                    if (cpt == 2) {         // two cells per thread, 4-byte words
                        const long long segs = interiorRows * (lists ? kTileCells / 2 : L.nz / 2);
                        const unsigned blocks = (unsigned)((segs + kBlock - 1) / kBlock);
                        vecRowStepKernel<S, ODD, STATS, EXT, 2><<<blocks, kBlock, 0, s>>>(L, pl, d, p, acc, segs);
                    } else if (cpt == 4) {  // four cells per thread, 8-byte vectors
                        const long long segs = interiorRows * (lists ? kTileCells / 4 : L.nz / 4);
                        const unsigned blocks = (unsigned)((segs + kBlock - 1) / kBlock);
                        vecRowStepKernel<S, ODD, STATS, EXT, 4><<<blocks, kBlock, 0, s>>>(L, pl, d, p, acc, segs);
                    } else {
                        const long long segs = interiorRows * (lists ? kTileCells / 8 : L.nz / 8);
                        const unsigned blocks = (unsigned)((segs + kBlock - 1) / kBlock);
                        vecRowStepKernel<S, ODD, STATS, EXT, 8><<<blocks, kBlock, 0, s>>>(L, pl, d, p, acc, segs);
                    }
                    ++launched;
                }
            } else if (pairedRows(L)) {
                Planes<S> pl;
                Deltas d;
                for (int i = 0; i < 19; ++i) {
                    pl.p[i] = static_cast<S*>(L.pop) + (long long)i * L.stride;
                    d.d[i] = cdir(i, 0) * L.ny * L.nz + cdir(i, 1) * L.nz + cdir(i, 2);
                }
                if constexpr (sizeof(S) == 2) {
                    const int pairs = L.nz / 2;
                    int tpb = (pairs + 31) / 32 * 32;
                    tpb = tpb < kBlock ? tpb : kBlock;
                    if (lists) tpb = kBlock;
                    const dim3 g = interiorGrid((pairs + tpb - 1) / tpb, kBlock / (kTileCells / 2));
                    pairRowStepKernel<S, ODD, STATS, EXT><<<g, tpb, 0, s>>>(L, pl, d, p, acc);
                    ++launched;
                }
            } else {
                Planes<S> pl;
                Deltas d;
                for (int i = 0; i < 19; ++i) {
                    pl.p[i] = static_cast<S*>(L.pop) + (long long)i * L.stride;
                    d.d[i] = cdir(i, 0) * L.ny * L.nz + cdir(i, 1) * L.nz + cdir(i, 2);
                }
                // one block per row segment of cells * threads cells; short rows get
                // fewer threads so that every thread owns `cells` live cells
                constexpr int NC = RowShape<S>::cells;
                int tpb = ((L.nz + NC - 1) / NC + 31) / 32 * 32;
                tpb = tpb < kBlock ? tpb : kBlock;
                if (lists) tpb = kBlock;
                rowStepKernel<S, ODD, STATS, EXT><<<interiorGrid((L.nz + tpb * NC - 1) / (tpb * NC), kBlock / kTileCells), tpb, 0, s>>>(L, pl, d, p,
                                                                                                        acc);
                ++launched;
            }
        };
        // interior-row tiles next to dropped blocks: the one-cell row kernel
        // with each cell's mask of neighbours outside the lattice, on the
        // border stream beside the interior kernel
        auto masked = [&]() {
            if (!lists || L.nMasked == 0) return;
            Planes<S> pl;
            Deltas d;
            for (int i = 0; i < 19; ++i) {
                pl.p[i] = static_cast<S*>(L.pop) + (long long)i * L.stride;
                d.d[i] = cdir(i, 0) * L.ny * L.nz + cdir(i, 1) * L.nz + cdir(i, 2);
            }
            const int blocks = (L.nMasked + kBlock / kTileCells - 1) / (kBlock / kTileCells);
            const unsigned gy = (unsigned)(blocks < 65535 ? blocks : 65535);
            rowStepKernel<S, ODD, STATS, EXT, true><<<dim3(1u, gy, (unsigned)((blocks + gy - 1) / gy)), kBlock, 0, es>>>(
                L, pl, d, p, acc);
            ++launched;
        };
        auto border = [&]() {
            if (edgeRows == 0 || slab) return;
            // rows, or blocks of kBlock / kTileCells tiles of the general-tile list
            const int blocks = lists ? (edgeRows + kBlock / kTileCells - 1) / (kBlock / kTileCells) : edgeRows;
            const int gy = blocks < 65535 ? blocks : 65535;
            dim3 g(lists ? 1u : (unsigned)((L.nz + kBlock - 1) / kBlock), (unsigned)gy, (unsigned)((blocks + gy - 1) / gy));
            if (L.sparse)
                edgeRowStepKernel<S, ODD, STATS, EXT, true><<<g, kBlock, 0, es>>>(L, p, acc, edgeRows);
            else
                edgeRowStepKernel<S, ODD, STATS, EXT, false><<<g, kBlock, 0, es>>>(L, p, acc, edgeRows);
            ++launched;
        };
        if (interiorFirst) {
            interior();
            masked();
            border();
        } else {
            border();
            interior();
            masked();
        }
        if (es != s) {   // join: the next step waits for both kernels
            if (cudaEventRecord(side->join, es) != cudaSuccess || cudaStreamWaitEvent(s, side->join, 0) != cudaSuccess)
                cudaStreamSynchronize(es);
        }
        return launched;
    }

};

// The border rows of the x-slab [x0, x1] of one AA step: whole planes x = 0
// and x = nx - 1 where the slab holds them, rows y = 0 and y = ny - 1 of its
// other planes (grid.y = rows: the planes' rows first, then two rows per
// interior plane), with the general addressing.  The slab's interior rows
// take the interior-row kernels (stepSplit over xRow0, xRows); slabs of a
// step launched separately beside host transfers (plbgpu_run_host).  Each
// slot is read and written by one cell per step, so the slabs of a step may
// run in any order once their inputs are final.
template <typename S, bool ODD, bool STATS, bool EXT>
__global__ void __launch_bounds__(128) slabBorderKernel(DevLattice L, StepParams<typename StoreT<S>::R> P,
                                                        StatsAcc* acc, int x0, int x1) {
    using R = typename StoreT<S>::R;
    const int z = blockIdx.x * blockDim.x + threadIdx.x;
    const int lo = x0 == 0 ? 1 : 0, hi = x1 == L.nx - 1 ? 1 : 0;
    int r = blockIdx.y, x, y;
    if (r < lo * L.ny) {
        x = 0; y = r;
    } else if ((r -= lo * L.ny) < hi * L.ny) {
        x = L.nx - 1; y = r;
    } else {
        r -= hi * L.ny;
        x = x0 + lo + (r >> 1);
        y = (r & 1) ? L.ny - 1 : 0;
    }
    R rhoBar = R(0), uSqr = R(0);
    bool g = false;
    if (z < L.nz) g = processCellGeneral<S, ODD, STATS, EXT, false>(L, P, x, y, z, acc, rhoBar, uSqr);
    accumulateStats<STATS>(g, (double)rhoBar, (double)uSqr, acc, L.status);
}

template <typename S, bool ODD, bool STATS, bool EXT>
int slabSplit(const DevLattice& L, const StepParams<typename StoreT<S>::R>& p, StatsAcc* acc, int x0, int x1,
              cudaStream_t s, const SideStream* side) {
    constexpr int kBlock = 128;
    int launched = 0;
    const int lo = x0 == 0 ? 1 : 0, hi = x1 == L.nx - 1 ? 1 : 0;
    const int a = x0 + lo, b = x1 - hi;          // the slab's planes with interior rows
    const int rows = (lo + hi) * L.ny + 2 * (b - a + 1);
    // the border rows beside the interior rows, on the side stream
    cudaStream_t es = s;
    if (side && b >= a && cudaEventRecord(side->fork, s) == cudaSuccess &&
        cudaStreamWaitEvent(side->stream, side->fork, 0) == cudaSuccess)
        es = side->stream;
    if (rows > 0) {
        const dim3 g((unsigned)((L.nz + kBlock - 1) / kBlock), (unsigned)rows, 1u);
        slabBorderKernel<S, ODD, STATS, EXT><<<g, kBlock, 0, es>>>(L, p, acc, x0, x1);
        ++launched;
    }
    if (b >= a) {
        DevLattice Ls = L;
        Ls.xRow0 = a - 1;
        Ls.xRows = b - a + 1;
        launched += StepLaunch<S>::template stepSplit<ODD, STATS, EXT>(Ls, p, acc, s, nullptr, true);
    }
    if (es != s) {   // join: the next launch on s waits for both kernels
        if (cudaEventRecord(side->join, es) != cudaSuccess || cudaStreamWaitEvent(s, side->join, 0) != cudaSuccess)
            cudaStreamSynchronize(es);
    }
    return launched;
}

template <typename S, bool ODD>
int slabParity(const DevLattice& L, bool stats, const StepParams<typename StoreT<S>::R>& p, StatsAcc* acc, int x0,
               int x1, cudaStream_t s, const SideStream* side) {
    if (p.external)
        return stats ? slabSplit<S, ODD, true, true>(L, p, acc, x0, x1, s, side)
                     : slabSplit<S, ODD, false, true>(L, p, acc, x0, x1, s, side);
    return stats ? slabSplit<S, ODD, true, false>(L, p, acc, x0, x1, s, side)
                 : slabSplit<S, ODD, false, false>(L, p, acc, x0, x1, s, side);
}

template <typename S, bool ODD>
int stepParity(const DevLattice& L, bool stats, const StepParams<typename StoreT<S>::R>& p, StatsAcc* acc,
               cudaStream_t s, const SideStream* side) {
    if (p.external)
        return stats ? StepLaunch<S>::template stepSplit<ODD, true, true>(L, p, acc, s, side)
                     : StepLaunch<S>::template stepSplit<ODD, false, true>(L, p, acc, s, side);
    return stats ? StepLaunch<S>::template stepSplit<ODD, true, false>(L, p, acc, s, side)
                 : StepLaunch<S>::template stepSplit<ODD, false, false>(L, p, acc, s, side);
}

}  // namespace plbgpu
