// The Palabos co-processor adapter (include/plbgpu_coprocessor3d.hh) driven end
// to end through the reference's own co-processor wiring, against the
// reference's example co-processor (D3Q19ExampleCoProcessor3D, which runs
// each pure-BGK block as a BlockLattice3D on the CPU:
// coProcessors/coProcessor3D.hh:36-76).
//
// Both runs build the same multi-block lattice (2 x 2 x 1 blocks, BGK), then
// call initiateCoProcessors (one co-processor domain per block, envelope box
// included), transferToCoProcessors, MultiBlockLattice3D::collideAndStream
// (which hands every block to the co-processor) and transferFromCoProcessors
// (coProcessors/coProcessorCommunication3D.hh:34-125,
// multiBlock/multiBlockLattice3D.hh:318-357).  The only difference is the
// object global::defaultCoProcessor3D<T>() returns -- the one place a Palabos
// maintainer changes to select the GPU (coProcessor3D.h:178-186): here an
// explicit specialization returns whichever co-processor the run selects.
//
// Prints, per lattice type, the largest population difference between the
// two runs and the number of co-processor domains used.
#include "parallelism/headers3D.h"
#include "parallelism/headers3D.hh"
#include "latticeBoltzmann/headers3D.h"
#include "latticeBoltzmann/headers3D.hh"
#include "core/headers3D.h"
#include "core/headers3D.hh"
#include "basicDynamics/headers3D.h"
#include "basicDynamics/headers3D.hh"
#include "atomicBlock/headers3D.h"
#include "atomicBlock/headers3D.hh"
#include "multiBlock/headers3D.h"
#include "multiBlock/headers3D.hh"
#include "dataProcessors/headers3D.h"
#include "dataProcessors/headers3D.hh"
#include "coProcessors/headers3D.h"
#include "coProcessors/headers3D.hh"

#include "plbgpu_coprocessor3d.hh"

#include <cmath>
#include <cstdio>
#include <vector>

namespace sel {
plb::CoProcessor3D<double>* cpDouble = 0;
plb::CoProcessor3D<float>* cpFloat = 0;
}  // namespace sel

namespace plb {
namespace global {
template <>
inline CoProcessor3D<double>& defaultCoProcessor3D<double>() { return *sel::cpDouble; }
template <>
inline CoProcessor3D<float>& defaultCoProcessor3D<float>() { return *sel::cpFloat; }
}  // namespace global
}  // namespace plb

using namespace plb;
typedef descriptors::D3Q19Descriptor<double> DD;

template <typename T>
void select(CoProcessor3D<T>& cp);
template <>
void select<double>(CoProcessor3D<double>& cp) { sel::cpDouble = &cp; }
template <>
void select<float>(CoProcessor3D<float>& cp) { sel::cpFloat = &cp; }

// nsteps collide-and-stream steps of a 20 x 16 x 12 lattice in 2 x 2 x 1 blocks
// on the given co-processor; returns the populations of every cell.
template <typename T>
std::vector<double> run(CoProcessor3D<T>& cp, int nsteps, int* domains) {
    select<T>(cp);
    const plint nx = 20, ny = 16, nz = 12;
    const T omega = (T)1.3;
    DefaultMultiBlockPolicy3D& policy = defaultMultiBlockPolicy3D();
    // The serial thread attribution ignores co-processor handles (every block
    // reports handle 0 and hasCoProcessors() is false: threadAttribution.h:60-62);
    // only the explicit attribution of MPI builds keeps them, so the blocks
    // are attributed explicitly to this process.
    ExplicitThreadAttribution* attribution = new ExplicitThreadAttribution();
    for (plint b = 0; b < 4; ++b) attribution->addBlock(b, 0);
    MultiBlockManagement3D management(createRegularDistribution3D(nx, ny, nz, 2, 2, 1), attribution, 1);
    MultiBlockLattice3D<T, descriptors::D3Q19Descriptor> lattice(
        management, policy.getBlockCommunicator(), policy.getCombinedStatistics(),
        policy.template getMultiCellAccess<T, descriptors::D3Q19Descriptor>(),
        new BGKdynamics<T, descriptors::D3Q19Descriptor>(omega));
    // a non-uniform initial flow: three boxes at equilibrium with different
    // densities and velocities
    initializeAtEquilibrium(lattice, lattice.getBoundingBox(), (T)1, Array<T, 3>((T)0.02, (T)0.01, (T)-0.01));
    initializeAtEquilibrium(lattice, Box3D(3, 11, 2, 9, 1, 7), (T)1.01, Array<T, 3>((T)-0.03, (T)0.02, (T)0.015));
    initializeAtEquilibrium(lattice, Box3D(12, 17, 6, 14, 4, 10), (T)0.995, Array<T, 3>((T)0.01, (T)-0.025, (T)0.03));
    lattice.initialize();
    initiateCoProcessors(lattice, BGKdynamics<T, descriptors::D3Q19Descriptor>(omega).getId(), false);
    transferToCoProcessors(lattice);
    for (int s = 0; s < nsteps; ++s) lattice.collideAndStream();
    transferFromCoProcessors(lattice);
    int handles = 0;
    ThreadAttribution const& ta = lattice.getMultiBlockManagement().getThreadAttribution();
    for (plint b = 0; b < 4 && ta.hasCoProcessors(); ++b)
        if (ta.getCoProcessorHandle(b) == (int)b) ++handles;   // one domain per block, in block order
    *domains = handles;
    std::vector<double> out;
    for (plint x = 0; x < nx; ++x)
        for (plint y = 0; y < ny; ++y)
            for (plint z = 0; z < nz; ++z) {
                Cell<T, descriptors::D3Q19Descriptor>& cell = lattice.get(x, y, z);
                for (int i = 0; i < 19; ++i) out.push_back((double)cell[i]);
            }
    return out;
}

template <typename T>
void compare(const char* name, int nsteps) {
    D3Q19ExampleCoProcessor3D<T> reference;
    plbgpu::GpuD3Q19CoProcessor3D<T> adapter(0);
    int dRef = 0, dAd = 0;
    std::vector<double> a = run<T>(reference, nsteps, &dRef);
    std::vector<double> b = run<T>(adapter, nsteps, &dAd);
    double maxDiff = 0., maxAbs = 0.;
    for (size_t i = 0; i < a.size(); ++i) {
        maxDiff = std::max(maxDiff, std::fabs(a[i] - b[i]));
        maxAbs = std::max(maxAbs, std::fabs(a[i]));
    }
    std::printf("%s domains=%d/%d cells=%zu maxdiff=%.17g maxabs=%.17g\n", name, dRef, dAd, a.size() / 19, maxDiff,
                maxAbs);
}

int main(int argc, char** argv) {
    plbInit(&argc, &argv);
    compare<double>("double", 7);
    compare<float>("float", 7);
    return 0;
}
