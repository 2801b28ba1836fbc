// Mirror of a Palabos lattice on the GPU library.  Include after the Palabos
// headers (it names plb::MultiBlockLattice3D, plb::Cell, plb::Box3D and
// plb::meta::dynamicsRegistration) and after plbgpu.hpp.
//
//   plb::MultiBlockLattice3D<double, D3Q19Descriptor> lattice(...);   // built as usual
//   ... defineDynamics, boundary conditions, initializeAtEquilibrium, lattice.initialize() ...
//   plbgpu::Context ctx(0);
//   plbgpu::PalabosDescription d = plbgpu::describe(lattice);        // host only
//   plbgpu::Lattice3D gpu(ctx, d.nx, d.ny, d.nz, d.omega, PLBGPU_FP64, d.rho0, d.bbRho);
//   plbgpu::upload(d, gpu);
//   gpu.collideAndStream(1000);
//   plbgpu::download(gpu, lattice);                                   // populations back
//
// describe() reads every cell's dynamics through the reference's registry of
// dynamics names (core/dynamicsIdentifiers.h:53-104) and turns it into the
// library's one-byte kinds:
//   "BGK", "BGK_ExternalForce_Guo", "BGK_Incompressible", "BounceBack",
//   "MomentumExchangeBounceBack", "NoDynamics"                (basic dynamics)
//   "Boundary_RegularizedVelocity_d_o", "Boundary_RegularizedDensity_d_o",
//   "Boundary_ZouHeVelocity_d_o", "Boundary_ZouHePressure_d_o"  (faces around BGK)
//   "Boundary_StoreVelocity"  (edges and corners of a velocity box; which one
//                              follows from the cell's place on the bounding box)
// and the values the GPU keeps per cell: the stored wall velocity
// (computeVelocity) of velocity boundaries, the stored density (computeDensity)
// of pressure boundaries, the force of a forced descriptor, and the
// populations (f-bar).  A dynamics it cannot map makes describe() throw.
#ifndef PLBGPU_PALABOS3D_HH
#define PLBGPU_PALABOS3D_HH

#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "plbgpu.hpp"

namespace plbgpu {

struct PalabosDescription {
    int nx = 0, ny = 0, nz = 0;
    bool periodic[3] = {false, false, false};
    double omega = 1.0, rho0 = 1.0, bbRho = 1.0;
    bool forced = false;
    std::vector<uint8_t> kinds;   // n, z fastest
    std::vector<double> bcval;    // 3n: wall velocity, or density in component 0
    std::vector<double> force;    // 3n when forced
    std::vector<double> f;        // 19n f-bar
};

namespace detail {

inline bool startsWith(const std::string& s, const std::string& p) { return s.compare(0, p.size(), p) == 0; }

// "…_<direction>_<orientation>" -> 2*direction + (orientation > 0)
inline int faceSuffix(const std::string& name, const std::string& prefix) {
    const std::string rest = name.substr(prefix.size());
    const size_t u = rest.find('_');
    if (u == std::string::npos) throw std::runtime_error("unexpected boundary dynamics name " + name);
    const int dir = std::atoi(rest.substr(0, u).c_str());
    const int ori = std::atoi(rest.substr(u + 1).c_str());
    return 2 * dir + (ori > 0 ? 1 : 0);
}

// Edge or corner kind of a stored-velocity cell from its place on the box.
inline int surfaceKind(int x, int y, int z, int nx, int ny, int nz) {
    const int p[3] = {x, y, z}, n[3] = {nx, ny, nz};
    int side[3], count = 0;
    for (int a = 0; a < 3; ++a) {
        side[a] = p[a] == 0 ? -1 : (p[a] == n[a] - 1 ? 1 : 0);
        count += side[a] != 0;
    }
    if (count == 3) return PLBGPU_VELOCITY_CORNER + 4 * (side[0] > 0) + 2 * (side[1] > 0) + (side[2] > 0);
    if (count == 2) {
        const int plane = !side[0] ? 0 : (!side[1] ? 1 : 2);
        return PLBGPU_VELOCITY_EDGE + 4 * plane + 2 * (side[(plane + 1) % 3] > 0) + (side[(plane + 2) % 3] > 0);
    }
    throw std::runtime_error("a stored-velocity cell that is not on an edge or corner of the lattice");
}

}  // namespace detail

// The kind of one dynamics name (position needed for stored-velocity cells).
inline int kindOfDynamics(const std::string& name, int x, int y, int z, int nx, int ny, int nz) {
    using detail::faceSuffix;
    using detail::startsWith;
    if (name == "BGK") return PLBGPU_BGK;
    if (name == "BGK_ExternalForce_Guo") return PLBGPU_GUO;
    if (name == "BGK_Incompressible") return PLBGPU_INCBGK;
    if (name == "BounceBack") return PLBGPU_BOUNCEBACK;
    if (name == "MomentumExchangeBounceBack") return PLBGPU_MOMENTUM_EXCHANGE;
    if (name == "NoDynamics") return PLBGPU_NODYNAMICS;
    if (startsWith(name, "Boundary_RegularizedVelocity_"))
        return PLBGPU_REG_VELOCITY + faceSuffix(name, "Boundary_RegularizedVelocity_");
    if (startsWith(name, "Boundary_RegularizedDensity_"))
        return PLBGPU_REG_PRESSURE + faceSuffix(name, "Boundary_RegularizedDensity_");
    if (startsWith(name, "Boundary_ZouHeVelocity_"))
        return PLBGPU_ZOUHE_VELOCITY + faceSuffix(name, "Boundary_ZouHeVelocity_");
    if (startsWith(name, "Boundary_ZouHePressure_"))
        return PLBGPU_ZOUHE_PRESSURE + faceSuffix(name, "Boundary_ZouHePressure_");
    if (name == "Boundary_StoreVelocity") return detail::surfaceKind(x, y, z, nx, ny, nz);
    throw std::runtime_error("dynamics '" + name + "' has no GPU kind");
}

// Read a Palabos lattice (MultiBlockLattice3D<double, D3Q19 or ForcedD3Q19>).
// rho0 is the IncBGK reference density (its dynamics keeps only 1/rho0).
template <template <typename U> class Descriptor>
PalabosDescription describe(plb::MultiBlockLattice3D<double, Descriptor>& lattice, double rho0 = 1.0) {
    typedef Descriptor<double> D;
    PalabosDescription d;
    const plb::Box3D box = lattice.getBoundingBox();
    d.nx = (int)box.getNx();
    d.ny = (int)box.getNy();
    d.nz = (int)box.getNz();
    for (int a = 0; a < 3; ++a) d.periodic[a] = lattice.periodicity().get(a);
    d.rho0 = rho0;
    d.forced = D::ExternalField::sizeOfForce == 3;
    const size_t n = (size_t)d.nx * d.ny * d.nz;
    d.kinds.assign(n, PLBGPU_BGK);
    d.bcval.assign(3 * n, 0.);
    d.f.assign(19 * n, 0.);
    if (d.forced) d.force.assign(3 * n, 0.);
    bool haveOmega = false, haveBb = false;
    for (int x = 0; x < d.nx; ++x)
        for (int y = 0; y < d.ny; ++y)
            for (int z = 0; z < d.nz; ++z) {
                const size_t id = ((size_t)x * d.ny + y) * d.nz + z;
                plb::Cell<double, Descriptor>& cell = lattice.get(box.x0 + x, box.y0 + y, box.z0 + z);
                const std::string name =
                    plb::meta::dynamicsRegistration<double, Descriptor>().getName(cell.getDynamics().getId());
                const int k = kindOfDynamics(name, x, y, z, d.nx, d.ny, d.nz);
                if (k >= PLBGPU_REG_VELOCITY) {   // boundary dynamics: the GPU runs them around BGK
                    const std::string base = plb::meta::dynamicsRegistration<double, Descriptor>().getName(
                        dynamic_cast<plb::CompositeDynamics<double, Descriptor>&>(cell.getDynamics())
                            .getBaseDynamics()
                            .getId());
                    if (base != "BGK") throw std::runtime_error(name + " around '" + base + "' has no GPU kind");
                }
                d.kinds[id] = (uint8_t)k;
                for (int i = 0; i < 19; ++i) d.f[19 * id + i] = cell[i];
                if (d.forced) {
                    const double* F = cell.getExternal(D::ExternalField::forceBeginsAt);
                    for (int a = 0; a < 3; ++a) d.force[3 * id + a] = F[a];
                }
                const bool velocity = (k >= PLBGPU_REG_VELOCITY && k < PLBGPU_REG_PRESSURE) ||
                                      (k >= PLBGPU_ZOUHE_VELOCITY && k < PLBGPU_ZOUHE_PRESSURE) ||
                                      k >= PLBGPU_VELOCITY_EDGE;
                const bool pressure = (k >= PLBGPU_REG_PRESSURE && k < PLBGPU_ZOUHE_VELOCITY) ||
                                      (k >= PLBGPU_ZOUHE_PRESSURE && k < PLBGPU_VELOCITY_EDGE);
                if (velocity) {
                    plb::Array<double, 3> u;
                    cell.computeVelocity(u);   // the stored wall velocity
                    for (int a = 0; a < 3; ++a) d.bcval[3 * id + a] = u[a];
                } else if (pressure) {
                    d.bcval[3 * id] = cell.computeDensity();   // the stored density
                }
                if (k == PLBGPU_BOUNCEBACK || k == PLBGPU_MOMENTUM_EXCHANGE) {
                    const double rho = cell.computeDensity();
                    if (haveBb && rho != d.bbRho)
                        throw std::runtime_error("bounce-back cells with different densities");
                    d.bbRho = rho;
                    haveBb = true;
                }
                if (k == PLBGPU_BGK || k == PLBGPU_GUO || k == PLBGPU_INCBGK || k >= PLBGPU_REG_VELOCITY) {
                    const double om = cell.getDynamics().getOmega();
                    if (haveOmega && om != d.omega) throw std::runtime_error("cells with different omega");
                    d.omega = om;
                    haveOmega = true;
                }
            }
    return d;
}

// Configure a GPU lattice of the same size from a description.
inline void upload(const PalabosDescription& d, Lattice3D& gpu) {
    const Box all = gpu.boundingBox();
    gpu.setParameters(d.omega, d.rho0, d.bbRho);
    gpu.periodicity(d.periodic[0], d.periodic[1], d.periodic[2]);
    gpu.setKinds(all, d.kinds);
    bool values = false, mebb = false, guo = false;
    for (uint8_t k : d.kinds) {
        values |= k >= PLBGPU_REG_VELOCITY;
        mebb |= k == PLBGPU_MOMENTUM_EXCHANGE;
        guo |= k == PLBGPU_GUO;
    }
    if (values) gpu.setBoundaryVelocity(all, d.bcval);
    if (guo && d.forced) gpu.setExternalVector(all, d.force);
    if (mebb) gpu.initializeMomentumExchange();
    gpu.send(all, d.f);
}

// Populations back into the Palabos lattice.
template <template <typename U> class Descriptor>
void download(const Lattice3D& gpu, plb::MultiBlockLattice3D<double, Descriptor>& lattice) {
    const plb::Box3D box = lattice.getBoundingBox();
    std::vector<double> f = gpu.receive(gpu.boundingBox());
    const int nx = (int)box.getNx(), ny = (int)box.getNy(), nz = (int)box.getNz();
    for (int x = 0; x < nx; ++x)
        for (int y = 0; y < ny; ++y)
            for (int z = 0; z < nz; ++z) {
                const size_t id = ((size_t)x * ny + y) * nz + z;
                plb::Cell<double, Descriptor>& cell = lattice.get(box.x0 + x, box.y0 + y, box.z0 + z);
                for (int i = 0; i < 19; ++i) cell[i] = f[19 * id + i];
            }
}

}  // namespace plbgpu

#endif  // PLBGPU_PALABOS3D_HH
