// Compiles the Palabos co-processor adapter (include/plbgpu_coprocessor3d.hh)
// against the reference's own headers and library, and drives it through the
// reference's co-processor wiring: initiateCoProcessors, transferTo/From and
// MultiBlockLattice3D::collideAndStream.  Without a GPU, addDomain fails
// cleanly (returns 0) and the lattice keeps running on the CPU path.
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

#include <cstdio>

using namespace plb;

int main(int argc, char** argv) {
    plbInit(&argc, &argv);
    plbgpu::GpuD3Q19CoProcessor3D<double> gpu(0);
    int handle = -1;
    int added = gpu.addDomain(10, 8, 6, 1.2, handle);
    std::printf("addDomain=%d context=%s\n", added, gpu.context() ? "yes" : "no");
    MultiBlockLattice3D<double, descriptors::D3Q19Descriptor> lattice(
        8, 8, 8, new BGKdynamics<double, descriptors::D3Q19Descriptor>(1.2));
    initializeAtEquilibrium(lattice, lattice.getBoundingBox(), 1.0, Array<double, 3>(0.01, 0., 0.));
    lattice.initialize();
    lattice.collideAndStream();
    std::printf("energy=%.12e\n", computeAverageEnergy(lattice));
    return 0;
}
