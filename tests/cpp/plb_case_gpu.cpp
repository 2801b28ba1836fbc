// GPU counterpart of oracle/ref_drivers/plb_case.cpp: reads the same case
// file, builds the lattice through the C++ front end (include/plbgpu.hpp),
// runs collideAndStream() and writes the same result file, so that a test can
// compare it with the reference driver's golden output.
//
//   plb_case_gpu <case-file> <result-file>
#include <cstdio>
#include <vector>

#include "../../oracle/ref_drivers/common.h"
#include "plbgpu.hpp"

using namespace refcase;

template <typename V>
static void wr(FILE* f, const V* p, size_t n) {
    if (std::fwrite(p, sizeof(V), n, f) != n) die("short write");
}

int main(int argc, char** argv) {
    if (argc != 3) die("usage: plb_case_gpu <case-file> <result-file>");
    Case c = readCase(argv[1]);
    plbgpu::Context ctx(0);
    plbgpu::Lattice3D lattice(ctx, c.nx, c.ny, c.nz, c.omega, PLBGPU_FP64, c.rho0, c.bbRho);
    lattice.periodicity(c.periodic[0], c.periodic[1], c.periodic[2]);
    const plbgpu::Box all = lattice.boundingBox();
    lattice.setKinds(all, c.flags);
    bool faces = false, guo = false, mebb = false;
    for (uint8_t k : c.flags) {
        faces |= k >= K_REGVEL && k < K_NKINDS;
        guo |= k == K_GUO;
        mebb |= k == K_MEBB;
    }
    if (faces) lattice.setBoundaryVelocity(all, c.bcval);   // density of pressure faces in component 0
    if (guo) lattice.setExternalVector(all, c.force);
    if (mebb) lattice.initializeMomentumExchange();
    lattice.send(all, c.f0);
    if (!(c.options & OPT_NO_INITIALIZE)) lattice.initialize();
    std::vector<double> fInit = lattice.receive(all);

    struct Rec { int32_t step; double v[6]; };
    std::vector<Rec> recs;
    for (int s = 0; s < c.nsteps; ++s) {
        const bool take = c.statsEvery > 0 && (s + 1) % c.statsEvery == 0;
        lattice.collideAndStream(1, take);
        if (take) {
            std::vector<double> st = lattice.internalStatistics();
            Rec r;
            r.step = s + 1;
            for (int i = 0; i < 6; ++i) r.v[i] = st[i];
            recs.push_back(r);
        }
    }
    std::vector<double> fFinal = lattice.receive(all);
    double energy = lattice.computeAverageEnergy(), density = lattice.computeAverageDensity();

    FILE* f = std::fopen(argv[2], "wb");
    if (!f) die("cannot open result file");
    wr(f, "PLBRES01", 8);
    int32_t h[5] = {c.nx, c.ny, c.nz, c.nsteps, (int32_t)recs.size()};
    wr(f, h, 5);
    wr(f, fInit.data(), fInit.size());
    wr(f, fFinal.data(), fFinal.size());
    for (const Rec& r : recs) {
        wr(f, &r.step, 1);
        wr(f, r.v, 6);
    }
    double tail[2] = {energy, density};
    wr(f, tail, 2);
    std::fclose(f);
    return 0;
}
