// Golden-vector driver: builds one parity case through the reference's own
// construction API (MultiBlockLattice3D, defineDynamics, the on-lattice
// boundary-condition instantiators, initializeMomentumExchange), runs
// collideAndStream() for the requested number of steps and writes the f-bar
// arrays plus the reductions.  See common.h for the file formats.
//
//   plb_case <case-file> <result-file>
//
// Test infrastructure only; linked against the unmodified reference library.
#include "common.h"

#include <cstdlib>

#include "parallelism/headers3D.h"
#include "parallelism/headers3D.hh"
#include "latticeBoltzmann/headers3D.h"
#include "latticeBoltzmann/headers3D.hh"
#include "core/headers3D.h"
#include "core/headers3D.hh"
#include "basicDynamics/headers3D.h"
#include "basicDynamics/headers3D.hh"
#include "boundaryCondition/headers3D.h"
#include "boundaryCondition/headers3D.hh"
#include "atomicBlock/headers3D.h"
#include "atomicBlock/headers3D.hh"
#include "multiBlock/headers3D.h"
#include "multiBlock/headers3D.hh"
#include "algorithm/headers3D.h"
#include "algorithm/headers3D.hh"
#include "dataProcessors/headers3D.h"
#include "dataProcessors/headers3D.hh"
#include "io/headers3D.h"
#include "io/headers3D.hh"
#include "coProcessors/headers3D.h"
#include "coProcessors/headers3D.hh"
#include "offLattice/makeSparse3D.h"
#include "offLattice/makeSparse3D.hh"

// The library's Palabos mirror (host part only: no GPU call is made here).
#include "plbgpu_palabos3d.hh"

using namespace plb;
using namespace refcase;

namespace {

struct CellValueVelocity {
    const Case* c;
    void operator()(plint x, plint y, plint z, Array<double,3>& u) const {
        long i = c->idx((int)x, (int)y, (int)z);
        u[0] = c->bcval[3 * i]; u[1] = c->bcval[3 * i + 1]; u[2] = c->bcval[3 * i + 2];
    }
};

struct CellValueDensity {
    const Case* c;
    double operator()(plint x, plint y, plint z) const {
        return c->bcval[3 * c->idx((int)x, (int)y, (int)z)];
    }
};

// Maximal runs of one kind along an axis that keeps the box planar for the
// given face direction (the wrapped boundary processors require x0==x1,
// y0==y1 or z0==z1).
std::vector<Box3D> planarRuns(const Case& c, int kind, int direction) {
    std::vector<Box3D> runs;
    if (direction != 2) {
        for (int x = 0; x < c.nx; ++x)
            for (int y = 0; y < c.ny; ++y) {
                int z = 0;
                while (z < c.nz) {
                    if (c.flags[c.idx(x, y, z)] != kind) { ++z; continue; }
                    int z1 = z;
                    while (z1 + 1 < c.nz && c.flags[c.idx(x, y, z1 + 1)] == kind) ++z1;
                    runs.push_back(Box3D(x, x, y, y, z, z1));
                    z = z1 + 1;
                }
            }
    } else {
        for (int y = 0; y < c.ny; ++y)
            for (int z = 0; z < c.nz; ++z) {
                int x = 0;
                while (x < c.nx) {
                    if (c.flags[c.idx(x, y, z)] != kind) { ++x; continue; }
                    int x1 = x;
                    while (x1 + 1 < c.nx && c.flags[c.idx(x1 + 1, y, z)] == kind) ++x1;
                    runs.push_back(Box3D(x, x1, y, y, z, z));
                    x = x1 + 1;
                }
            }
    }
    return runs;
}

DotList3D dotsOfKind(const Case& c, int kind) {
    DotList3D dots;
    for (int x = 0; x < c.nx; ++x)
        for (int y = 0; y < c.ny; ++y)
            for (int z = 0; z < c.nz; ++z)
                if (c.flags[c.idx(x, y, z)] == kind) dots.addDot(Dot3D(x, y, z));
    return dots;
}

template<template<typename U> class D>
void addFace(OnLatticeBoundaryCondition3D<double,D>& bc, MultiBlockLattice3D<double,D>& lat,
             bool velocity, int dir, int ori, Box3D const& b) {
    if (velocity) {
        switch (dir * 2 + (ori > 0)) {
            case 0: bc.addVelocityBoundary0N(b, lat); break;
            case 1: bc.addVelocityBoundary0P(b, lat); break;
            case 2: bc.addVelocityBoundary1N(b, lat); break;
            case 3: bc.addVelocityBoundary1P(b, lat); break;
            case 4: bc.addVelocityBoundary2N(b, lat); break;
            case 5: bc.addVelocityBoundary2P(b, lat); break;
        }
    } else {
        switch (dir * 2 + (ori > 0)) {
            case 0: bc.addPressureBoundary0N(b, lat); break;
            case 1: bc.addPressureBoundary0P(b, lat); break;
            case 2: bc.addPressureBoundary1N(b, lat); break;
            case 3: bc.addPressureBoundary1P(b, lat); break;
            case 4: bc.addPressureBoundary2N(b, lat); break;
            case 5: bc.addPressureBoundary2P(b, lat); break;
        }
    }
}

// External velocity edge (plane, normal1, normal2) of the local regularized
// condition (boundaryCondition/boundaryInstantiator3D.h:76-98).
template<template<typename U> class D>
void addEdge(OnLatticeBoundaryCondition3D<double,D>& bc, MultiBlockLattice3D<double,D>& lat, int e,
             Box3D const& b) {
    switch (e) {
        case 0: bc.addExternalVelocityEdge0NN(b, lat); break;
        case 1: bc.addExternalVelocityEdge0NP(b, lat); break;
        case 2: bc.addExternalVelocityEdge0PN(b, lat); break;
        case 3: bc.addExternalVelocityEdge0PP(b, lat); break;
        case 4: bc.addExternalVelocityEdge1NN(b, lat); break;
        case 5: bc.addExternalVelocityEdge1NP(b, lat); break;
        case 6: bc.addExternalVelocityEdge1PN(b, lat); break;
        case 7: bc.addExternalVelocityEdge1PP(b, lat); break;
        case 8: bc.addExternalVelocityEdge2NN(b, lat); break;
        case 9: bc.addExternalVelocityEdge2NP(b, lat); break;
        case 10: bc.addExternalVelocityEdge2PN(b, lat); break;
        case 11: bc.addExternalVelocityEdge2PP(b, lat); break;
    }
}

// External velocity corner (xNormal, yNormal, zNormal)
// (boundaryCondition/boundaryInstantiator3D.h:126-141).
template<template<typename U> class D>
void addCorner(OnLatticeBoundaryCondition3D<double,D>& bc, MultiBlockLattice3D<double,D>& lat, int k, plint x,
               plint y, plint z) {
    switch (k) {
        case 0: bc.addExternalVelocityCornerNNN(x, y, z, lat); break;
        case 1: bc.addExternalVelocityCornerNNP(x, y, z, lat); break;
        case 2: bc.addExternalVelocityCornerNPN(x, y, z, lat); break;
        case 3: bc.addExternalVelocityCornerNPP(x, y, z, lat); break;
        case 4: bc.addExternalVelocityCornerPNN(x, y, z, lat); break;
        case 5: bc.addExternalVelocityCornerPNP(x, y, z, lat); break;
        case 6: bc.addExternalVelocityCornerPPN(x, y, z, lat); break;
        case 7: bc.addExternalVelocityCornerPPP(x, y, z, lat); break;
    }
}

template<typename V>
void wr(FILE* f, const V* p, size_t n) {
    if (std::fwrite(p, sizeof(V), n, f) != n) die("short write");
}

template<template<typename U> class D>
bool inLattice(MultiBlockLattice3D<double,D>& lat, int x, int y, int z) {
    return lat.getMultiBlockManagement().getSparseBlockStructure().locate(x, y, z) >= 0;
}

// Cells outside every block of a sparse lattice are written as zeros.
template<template<typename U> class D>
void dumpPopulations(MultiBlockLattice3D<double,D>& lat, const Case& c, std::vector<double>& out) {
    out.assign(c.n() * 19, 0.);
    for (int x = 0; x < c.nx; ++x)
        for (int y = 0; y < c.ny; ++y)
            for (int z = 0; z < c.nz; ++z) {
                if (!inLattice(lat, x, y, z)) continue;
                Cell<double,D>& cell = lat.get(x, y, z);
                for (int i = 0; i < 19; ++i) out[c.idx(x, y, z) * 19 + i] = cell[i];
            }
}

template<template<typename U> class D, class BulkDynamics>
int run(const Case& c, const char* outPath) {
    typedef MultiBlockLattice3D<double,D> Lattice;
    DefaultMultiBlockPolicy3D& policy = defaultMultiBlockPolicy3D();
    MultiBlockManagement3D dense(
        createRegularDistribution3D(c.nx, c.ny, c.nz, c.blocks[0], c.blocks[1], c.blocks[2]),
        policy.getThreadAttribution(), 1);
    const bool sparse = (c.options & OPT_SPARSE) != 0;
    MultiBlockManagement3D management(dense);
    if (sparse) {
        // computeSparseManagement (offLattice/makeSparse3D.hh:107-160) of the
        // case's int field on the same regular distribution.
        MultiScalarField3D<int> field(dense, policy.getBlockCommunicator(), policy.getCombinedStatistics(),
                                      policy.getMultiScalarAccess<int>(), 0);
        for (int x = 0; x < c.nx; ++x)
            for (int y = 0; y < c.ny; ++y)
                for (int z = 0; z < c.nz; ++z) field.get(x, y, z) = c.sparse[c.idx(x, y, z)];
        management = computeSparseManagement(field, 1);
    }
    Lattice lat(management, policy.getBlockCommunicator(), policy.getCombinedStatistics(),
                policy.template getMultiCellAccess<double,D>(),
                new BulkDynamics(c.omega));
    for (int a = 0; a < 3; ++a) lat.periodicity().toggle(a, c.periodic[a] != 0);

    // Bulk dynamics other than the background.
    DotList3D dots;
    dots = dotsOfKind(c, K_BGK);
    if (dots.getN() > 0) defineDynamics(lat, dots, new BGKdynamics<double,D>(c.omega));
    dots = dotsOfKind(c, K_INCBGK);
    if (dots.getN() > 0) defineDynamics(lat, dots, new IncBGKdynamics<double,D>(c.omega, c.rho0));
    dots = dotsOfKind(c, K_GUO);
    if (dots.getN() > 0) defineDynamics(lat, dots, new GuoExternalForceBGKdynamics<double,D>(c.omega));
    dots = dotsOfKind(c, K_BB);
    if (dots.getN() > 0) defineDynamics(lat, dots, new BounceBack<double,D>(c.bbRho));
    dots = dotsOfKind(c, K_NODYN);
    if (dots.getN() > 0) defineDynamics(lat, dots, new NoDynamics<double,D>(c.bbRho));

    Array<plint,3> forceIds;
    forceIds[0] = lat.internalStatSubscription().subscribeSum();
    forceIds[1] = lat.internalStatSubscription().subscribeSum();
    forceIds[2] = lat.internalStatSubscription().subscribeSum();
    dots = dotsOfKind(c, K_MEBB);
    bool haveMebb = dots.getN() > 0;
    if (haveMebb) defineDynamics(lat, dots, new MomentumExchangeBounceBack<double,D>(forceIds, c.bbRho));

    // Boundary cells: composite dynamics wrapped around a BGK base.
    OnLatticeBoundaryCondition3D<double,D>* reg = createLocalBoundaryCondition3D<double,D>();
    OnLatticeBoundaryCondition3D<double,D>* zh = createZouHeBoundaryCondition3D<double,D>();
    for (int k = K_REGVEL; k < K_EDGE; ++k) {
        dots = dotsOfKind(c, k);
        if (dots.getN() == 0) continue;
        defineDynamics(lat, dots, new BGKdynamics<double,D>(c.omega));
        int family = (k - K_REGVEL) / 6, sub = (k - K_REGVEL) % 6;
        int dir = sub / 2, ori = (sub % 2) ? 1 : -1;
        bool velocity = (family == 0 || family == 2);
        OnLatticeBoundaryCondition3D<double,D>& bc = (family < 2) ? *reg : *zh;
        std::vector<Box3D> runs = planarRuns(c, k, dir);
        for (size_t r = 0; r < runs.size(); ++r) {
            addFace(bc, lat, velocity, dir, ori, runs[r]);
            if (velocity) {
                CellValueVelocity fv = {&c};
                setBoundaryVelocity(lat, runs[r], fv);
            } else {
                CellValueDensity fd = {&c};
                setBoundaryDensity(lat, runs[r], fd);
            }
        }
    }
    // Edges and corners after every face, so that their finite-difference
    // processors run after the face processors, as setVelocityConditionOnBlockBoundaries
    // orders them (boundaryCondition/boundaryCondition3D.hh:65-163).
    for (int k = K_EDGE; k < K_NKINDS; ++k) {
        dots = dotsOfKind(c, k);
        if (dots.getN() == 0) continue;
        defineDynamics(lat, dots, new BGKdynamics<double,D>(c.omega));
        for (int x = 0; x < c.nx; ++x)
            for (int y = 0; y < c.ny; ++y)
                for (int z = 0; z < c.nz; ++z) {
                    if (c.flags[c.idx(x, y, z)] != k) continue;
                    Box3D b(x, x, y, y, z, z);
                    if (k < K_CORNER) addEdge(*reg, lat, k - K_EDGE, b);
                    else addCorner(*reg, lat, k - K_CORNER, x, y, z);
                    CellValueVelocity fv = {&c};
                    setBoundaryVelocity(lat, b, fv);
                }
    }
    if (haveMebb) initializeMomentumExchange(lat, lat.getBoundingBox());

    // Initial populations (and the Guo force field).
    for (int x = 0; x < c.nx; ++x)
        for (int y = 0; y < c.ny; ++y)
            for (int z = 0; z < c.nz; ++z) {
                if (!inLattice(lat, x, y, z)) continue;
                Cell<double,D>& cell = lat.get(x, y, z);
                long id = c.idx(x, y, z);
                for (int i = 0; i < 19; ++i) cell[i] = c.f0[id * 19 + i];
                if (c.forced) {
                    double* ext = cell.getExternal(0);
                    ext[0] = c.force[3 * id]; ext[1] = c.force[3 * id + 1]; ext[2] = c.force[3 * id + 2];
                }
            }
    if (!(c.options & OPT_NO_INITIALIZE)) lat.initialize();

    // With PLB_LOAD_STATE=<base>: the populations come from a saved state
    // (parallelIO::load of <base>.plb / <base>.dat, static content).
    if (const char* lpath = std::getenv("PLB_LOAD_STATE")) parallelIO::load(lpath, lat, false);
    // With PLB_LOAD_DYNAMIC_STATE=<plb>: parallelIO::load(plb, lattice, true) --
    // the dynamics objects are regenerated from the state, then the populations.
    if (const char* lpath = std::getenv("PLB_LOAD_DYNAMIC_STATE")) parallelIO::load(lpath, lat, true);

    std::vector<double> fInit, fFinal;
    dumpPopulations(lat, c, fInit);

    // With PLB_DESCRIBE=<path>: what plbgpu::describe() reads from the lattice
    // after initialize() -- kinds (uint8 N), values (float64 3N), force
    // (float64 3N, zeros without a forced descriptor), f-bar (float64 19N),
    // omega, bbRho.
    if (const char* dpath = std::getenv("PLB_DESCRIBE")) {
        plbgpu::PalabosDescription dsc = plbgpu::describe(lat, c.rho0);
        FILE* df = std::fopen(dpath, "wb");
        if (!df) die("cannot open description file");
        wr(df, dsc.kinds.data(), dsc.kinds.size());
        wr(df, dsc.bcval.data(), dsc.bcval.size());
        std::vector<double> force(dsc.forced ? dsc.force : std::vector<double>(3 * c.n(), 0.));
        wr(df, force.data(), force.size());
        wr(df, dsc.f.data(), dsc.f.size());
        double tail2[2] = {dsc.omega, dsc.bbRho};
        wr(df, tail2, 2);
        std::fclose(df);
    }

    // The external rho-bar / j form: the two processors of a lattice stepped
    // by executeInternalProcessors() instead of collideAndStream().
    const bool external = (c.options & OPT_EXTERNAL_RHOJ) != 0;
    std::auto_ptr<MultiScalarField3D<double> > rhoBarF;
    std::auto_ptr<MultiTensorField3D<double,3> > jF;
    if (external) {
        rhoBarF = generateMultiScalarField<double>(lat, 1);
        jF = generateMultiTensorField<double,3>(lat, 1);
        for (int a = 0; a < 3; ++a) {
            rhoBarF->periodicity().toggle(a, c.periodic[a] != 0);
            jF->periodicity().toggle(a, c.periodic[a] != 0);
        }
        for (int x = 0; x < c.nx; ++x)
            for (int y = 0; y < c.ny; ++y)
                for (int z = 0; z < c.nz; ++z) {
                    long id = c.idx(x, y, z);
                    rhoBarF->get(x, y, z) = c.rhoBar0[id];
                    Array<double,3>& jj = jF->get(x, y, z);
                    jj[0] = c.j0[3 * id]; jj[1] = c.j0[3 * id + 1]; jj[2] = c.j0[3 * id + 2];
                }
        rhoBarF->duplicateOverlaps(modif::staticVariables);
        jF->duplicateOverlaps(modif::staticVariables);
        std::vector<MultiBlock3D*> args;
        args.push_back(&lat);
        args.push_back(rhoBarF.get());
        args.push_back(jF.get());
        integrateProcessingFunctional(new ExternalRhoJcollideAndStream3D<double,D>(), lat.getBoundingBox(), args, 0);
        integrateProcessingFunctional(new BoxRhoBarJfunctional3D<double,D>(), lat.getBoundingBox(), args, 3);
    }

    struct Rec { int32_t step; double v[6]; };
    std::vector<Rec> recs;
    for (int s = 0; s < c.nsteps; ++s) {
        if (external) {
            lat.executeInternalProcessors();
            lat.evaluateStatistics();
            lat.incrementTime();
        } else {
            lat.collideAndStream();
        }
        if (c.statsEvery > 0 && (s + 1) % c.statsEvery == 0) {
            BlockStatistics const& st = lat.getInternalStatistics();
            Rec r;
            r.step = s + 1;
            r.v[0] = st.getAverage(LatticeStatistics::avRhoBar);
            r.v[1] = st.getAverage(LatticeStatistics::avUSqr);
            r.v[2] = st.getMax(LatticeStatistics::maxUSqr);
            for (int d = 0; d < 3; ++d) r.v[3 + d] = st.getSum(forceIds[d]);
            recs.push_back(r);
        }
    }
    dumpPopulations(lat, c, fFinal);
    double energy = computeAverageEnergy(lat);
    double density = computeAverageDensity(lat);
    if (c.options & OPT_SAVE_STATE) {   // <result without extension>_state.plb / .dat
        std::string base(outPath);
        const size_t slash = base.rfind('/'), dot = base.rfind('.');
        if (dot != std::string::npos && (slash == std::string::npos || dot > slash)) base.erase(dot);
        parallelIO::save(lat, base + "_state", false);
    }
    if (c.options & OPT_SAVE_DYNAMIC_STATE) {   // <result without extension>_dstate.plb / .dat
        std::string base(outPath);
        const size_t slash = base.rfind('/'), dot = base.rfind('.');
        if (dot != std::string::npos && (slash == std::string::npos || dot > slash)) base.erase(dot);
        parallelIO::save(lat, base + "_dstate", true);
    }
    if (c.options & OPT_SAVE_BINARY) {
        std::string base(outPath);
        saveBinaryBlock(lat, base + ".lattice");
        saveBinaryBlock(*computeDensity(lat), base + ".density");
        saveBinaryBlock(*computeVelocity(lat), base + ".velocity");
    }

    FILE* f = std::fopen(outPath, "wb");
    if (!f) die("cannot open result file");
    wr(f, "PLBRES01", 8);
    int32_t h[5] = {c.nx, c.ny, c.nz, c.nsteps, (int32_t)recs.size()};
    wr(f, h, 5);
    wr(f, fInit.data(), fInit.size());
    wr(f, fFinal.data(), fFinal.size());
    for (size_t i = 0; i < recs.size(); ++i) {
        wr(f, &recs[i].step, 1);
        wr(f, recs[i].v, 6);
    }
    double tail[2] = {energy, density};
    wr(f, tail, 2);
    if (sparse) {     // cells of the kept blocks
        std::vector<uint8_t> in(c.n());
        for (int x = 0; x < c.nx; ++x)
            for (int y = 0; y < c.ny; ++y)
                for (int z = 0; z < c.nz; ++z)
                    in[c.idx(x, y, z)] = management.getSparseBlockStructure().locate(x, y, z) >= 0 ? 1 : 0;
        wr(f, in.data(), in.size());
    }
    if (external) {   // the fields after the last BoxRhoBarJfunctional3D
        std::vector<double> rb(c.n()), jj(3 * c.n());
        for (int x = 0; x < c.nx; ++x)
            for (int y = 0; y < c.ny; ++y)
                for (int z = 0; z < c.nz; ++z) {
                    long id = c.idx(x, y, z);
                    rb[id] = rhoBarF->get(x, y, z);
                    Array<double,3> const& v = jF->get(x, y, z);
                    for (int d = 0; d < 3; ++d) jj[3 * id + d] = v[d];
                }
        wr(f, rb.data(), rb.size());
        wr(f, jj.data(), jj.size());
    }
    std::fclose(f);
    delete reg;
    delete zh;
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    plbInit(&argc, &argv);
    if (argc != 3) die("usage: plb_case <case-file> <result-file>");
    Case c = readCase(argv[1]);
    if (c.forced)
        return run<descriptors::ForcedD3Q19Descriptor,
                   GuoExternalForceBGKdynamics<double,descriptors::ForcedD3Q19Descriptor> >(c, argv[2]);
    return run<descriptors::D3Q19Descriptor,
               BGKdynamics<double,descriptors::D3Q19Descriptor> >(c, argv[2]);
}
