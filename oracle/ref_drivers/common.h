// Shared case-file format for the golden-vector drivers.
//
// These drivers are test infrastructure: they link the UNMODIFIED reference
// library (built by oracle/Makefile.ref from the reference sources) and are
// used only to produce golden fixtures under tests/golden/.  Nothing in the
// product links them.
//
// Case file (little endian), written by tests/golden/make_golden.py:
//   char[8]  "PLBCASE1"
//   int32    nx, ny, nz
//   int32    periodic_x, periodic_y, periodic_z
//   int32    forced            (1: ForcedD3Q19 descriptor, 0: D3Q19)
//   int32    blocks_x, blocks_y, blocks_z   (regular block decomposition)
//   int32    nsteps
//   int32    stats_every        (record stored statistics every k steps, 0 = never)
//   int32    options            (bit 0: do not call lattice.initialize())
//   float64  omega, rho0 (IncBGK reference density), bbRho
//   uint8    flags[N]           (kind per cell, x-major, z fastest)
//   float64  bcval[N*3]         (velocity for velocity faces, rho in [0] for pressure faces)
//   float64  force[N*3]         (Guo force, only read when forced)
//   float64  f0[N*19]           (initial f-bar, before lattice.initialize())
//   float64  rhoBar0[N], j0[N*3] (only with OPT_EXTERNAL_RHOJ: initial fields)
//   int32    sparse[N]           (only with OPT_SPARSE: the field of computeSparseManagement)
//
// Result file:
//   char[8]  "PLBRES01"
//   int32    nx, ny, nz, nsteps, nstat
//   float64  f_init[N*19]       (after lattice.initialize(): BC cells completed)
//   float64  f_final[N*19]      (after nsteps collideAndStream())
//   per recorded step k (nstat records): int32 step, float64 avRhoBar, avUSqr,
//                                         maxUSqr, drag[3]
//   float64  avgEnergy, avgDensity   (computeAverageEnergy / computeAverageDensity
//                                     over the bounding box after nsteps)
//   float64  rhoBar[N], j[N*3]   (only with OPT_EXTERNAL_RHOJ: the fields at the end)
//   uint8    inLattice[N]        (only with OPT_SPARSE: 1 for cells of kept blocks)
#ifndef PLB_REF_DRIVER_COMMON_H
#define PLB_REF_DRIVER_COMMON_H

#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <string>

namespace refcase {

// Cell kinds.  The same numbering is used by the oracle and the CUDA path.
enum Kind {
    K_BGK = 0, K_GUO = 1, K_INCBGK = 2, K_BB = 3, K_MEBB = 4, K_NODYN = 5,
    K_REGVEL = 6,     // 6..11  : 6 + 2*direction + (orientation>0)
    K_REGPRESS = 12,  // 12..17
    K_ZHVEL = 18,     // 18..23
    K_ZHPRESS = 24,   // 24..29
    K_EDGE = 30,      // 30..41 : 30 + 4*plane + 2*(normal1>0) + (normal2>0)
    K_CORNER = 42,    // 42..49 : 42 + 4*(xNormal>0) + 2*(yNormal>0) + (zNormal>0)
    K_NKINDS = 50
};

// Case options (header word 12).
enum {
    OPT_NO_INITIALIZE = 1,   // skip lattice.initialize() before the first step
    OPT_EXTERNAL_RHOJ = 2,   // step with ExternalRhoJcollideAndStream3D (level 0) and
                             // BoxRhoBarJfunctional3D (level 3) from the given fields
    OPT_SAVE_BINARY = 4,     // after the run, saveBinaryBlock of the lattice, of
                             // computeDensity and of computeVelocity into
                             // <result>.lattice / .density / .velocity
    OPT_SPARSE = 8,          // build the lattice on computeSparseManagement of the
                             // given int field over the regular block distribution
    OPT_SAVE_STATE = 16,     // after the run, parallelIO::save(lattice, <base>_state, false)
                             // with <base> the result path without its extension
    OPT_SAVE_DYNAMIC_STATE = 32  // after the run, parallelIO::save(lattice, <base>_dstate, true):
                                 // the state with dynamic content (serialized dynamics)
};

struct Case {
    int nx, ny, nz;
    int periodic[3];
    int forced;
    int blocks[3];
    int nsteps;
    int statsEvery;
    int options;
    double omega, rho0, bbRho;
    std::vector<uint8_t> flags;
    std::vector<double> bcval, force, f0, rhoBar0, j0;
    std::vector<int32_t> sparse;
    long n() const { return (long)nx * ny * nz; }
    long idx(int x, int y, int z) const { return ((long)x * ny + y) * nz + z; }
};

inline void die(const char* msg) {
    std::fprintf(stderr, "ref driver: %s\n", msg);
    std::exit(2);
}

template<typename V>
inline void rd(FILE* f, V* p, size_t n) {
    if (std::fread(p, sizeof(V), n, f) != n) die("short read");
}

inline Case readCase(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) die("cannot open case file");
    char magic[8];
    rd(f, magic, 8);
    if (std::memcmp(magic, "PLBCASE1", 8) != 0) die("bad case magic");
    Case c;
    int32_t h[13];
    rd(f, h, 13);
    c.nx = h[0]; c.ny = h[1]; c.nz = h[2];
    c.periodic[0] = h[3]; c.periodic[1] = h[4]; c.periodic[2] = h[5];
    c.forced = h[6];
    c.blocks[0] = h[7]; c.blocks[1] = h[8]; c.blocks[2] = h[9];
    c.nsteps = h[10]; c.statsEvery = h[11];
    c.options = h[12];
    double d[3];
    rd(f, d, 3);
    c.omega = d[0]; c.rho0 = d[1]; c.bbRho = d[2];
    long n = c.n();
    c.flags.resize(n); rd(f, c.flags.data(), n);
    c.bcval.resize(n * 3); rd(f, c.bcval.data(), n * 3);
    c.force.resize(n * 3); rd(f, c.force.data(), n * 3);
    c.f0.resize(n * 19); rd(f, c.f0.data(), n * 19);
    if (c.options & OPT_EXTERNAL_RHOJ) {
        c.rhoBar0.resize(n); rd(f, c.rhoBar0.data(), n);
        c.j0.resize(n * 3); rd(f, c.j0.data(), n * 3);
    }
    if (c.options & OPT_SPARSE) {
        c.sparse.resize(n); rd(f, c.sparse.data(), n);
    }
    std::fclose(f);
    return c;
}

}  // namespace refcase

#endif
