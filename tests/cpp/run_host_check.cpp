// plbgpu::Lattice3D::runHost (plbgpu_run_host) against the three calls it
// replaces -- send, collideAndStream, receive -- on a channel with a
// regularized velocity inlet, a pressure outlet, bounce-back walls and an
// obstacle, FP64.  The state must agree bit for bit, the statistics records
// to summation rounding.  Prints one line: "runhost cells=... maxabs=...
// maxdiff=... statsrel=... records=...".
#include <cmath>
#include <cstdio>
#include <vector>

#include "plbgpu.hpp"

namespace {

void build(plbgpu::Lattice3D& lat, int nx, int ny, int nz) {
    using plbgpu::Box;
    lat.defineDynamics(Box{0, nx - 1, 0, 0, 0, nz - 1}, PLBGPU_BOUNCEBACK);
    lat.defineDynamics(Box{0, nx - 1, ny - 1, ny - 1, 0, nz - 1}, PLBGPU_BOUNCEBACK);
    lat.defineDynamics(Box{0, nx - 1, 1, ny - 2, 0, 0}, PLBGPU_BOUNCEBACK);
    lat.defineDynamics(Box{0, nx - 1, 1, ny - 2, nz - 1, nz - 1}, PLBGPU_BOUNCEBACK);
    lat.defineDynamics(Box{9, 11, 4, 6, 4, 7}, PLBGPU_BOUNCEBACK);   // the obstacle
    const Box inlet{0, 0, 1, ny - 2, 1, nz - 2}, outlet{nx - 1, nx - 1, 1, ny - 2, 1, nz - 2};
    lat.addVelocityBoundary(inlet, 0, -1);
    lat.addPressureBoundary(outlet, 0, +1);
    lat.setBoundaryVelocity(inlet, 0.04, 0., 0.);
    lat.setBoundaryDensity(outlet, 1.0);
    lat.initializeAtEquilibrium(lat.boundingBox(), 1.0, 0.02, 0., 0.);
    lat.initialize();
}

}  // namespace

int main() {
    const int nx = 34, ny = 11, nz = 12, steps = 9, every = 4;
    plbgpu::Context ctx(0);
    plbgpu::Lattice3D a(ctx, nx, ny, nz, 1.7), b(ctx, nx, ny, nz, 1.7);
    build(a, nx, ny, nz);
    build(b, nx, ny, nz);
    a.collideAndStream(5, false);
    b.collideAndStream(5, false);
    const plbgpu::Box all = b.boundingBox();
    std::vector<double> f = b.receive(all);

    std::vector<double> fa = f;
    const std::vector<double> sa = a.runHost(fa, steps, every);

    b.send(all, f);
    std::vector<double> sb;
    for (int done = 0; done < steps;) {
        const int chunk = done + every <= steps ? every : steps - done;
        b.collideAndStream(chunk, true);
        const std::vector<double> s = b.internalStatistics();
        sb.insert(sb.end(), s.begin(), s.end());
        done += chunk;
    }
    const std::vector<double> fb = b.receive(all);

    double maxabs = 0., maxdiff = 0., statsrel = 0.;
    for (size_t i = 0; i < fb.size(); ++i) {
        maxabs = std::fmax(maxabs, std::fabs(fb[i]));
        maxdiff = std::fmax(maxdiff, std::fabs(fa[i] - fb[i]));
    }
    for (size_t i = 0; i < sb.size() && i < sa.size(); ++i)
        statsrel = std::fmax(statsrel, std::fabs(sa[i] - sb[i]) / std::fmax(1e-300, std::fabs(sb[i])));
    std::printf("runhost cells=%d maxabs=%.17g maxdiff=%.17g statsrel=%.3g records=%zu/%zu\n", nx * ny * nz, maxabs,
                maxdiff, statsrel, sa.size() / 7, sb.size() / 7);
    return 0;
}
