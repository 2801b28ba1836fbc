// Golden-vector driver for the voxelizer: the reference's own
// voxelize(mesh, domain, borderWidth) (offLattice/voxelizer.hh:106-141) on a
// triangle set given in lattice units.
//
//   plb_voxel --stl <file.stl> <flt|dbl> <result>
//   result: "PLBTRI01", int32 n, float64 triangles[n][3][3] -- what
//           TriangleSet<double>(file, precision) read (offLattice/triangleSet.hh:70-345)
//
//   plb_voxel --scale <file.stl> <resolution> <referenceDirection> <margin> <extraLayer> <result>
//   result: "PLBTRI01", as above -- the triangles of DEFscaledMesh(TriangleSet<double>(file, DBL),
//           resolution, referenceDirection, margin, extraLayer) in lattice units
//           (offLattice/triangleBoundary3D.hh:255-300, triangularSurfaceMesh.hh:1552-1575)
//
//   plb_voxel <case> <result>
//   case:   "PLBVOX01", int32 nx, ny, nz, borderWidth, nTriangles,
//           float64 triangles[nTriangles][3][3] (vertex, then x, y, z)
//   result: "PLBVXR01", int32 nx, ny, nz, then int32 flags[nx][ny][nz]
//           (z fastest): 1 outside, 2 outerBorder, 3 inside, 4 innerBorder
//
// The fork's voxelizer header pulls in its application headers
// (myheaders3D.hh), whose debug.h does not compile with g++ 13 (debug.h:265
// uses a template parameter in a function that is not a template), and
// palabos3D.hh pulls in the multigrid templates, which do not compile either
// (multiGrid/coarseGridProcessors3D.hh:159).  Neither is on the voxelizer's
// path: their include guards are defined here so they are skipped, and the
// one function the voxelizer takes from debug.h -- exHandler, its catch
// handler -- is declared below (it reports and aborts).  PLB_DEBUG is defined
// because the fork's triangleSet.hh declares a variable it uses
// (offLattice/triangleSet.hh:151) only in debug builds.
#define PLB_DEBUG
#define MYHEADERS3D_H
#define MYHEADERS3D_HH
#define DEBUG_HH
#define COARSE_GRID_PROCESSORS_3D_HH

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

namespace plb {
void exHandler(const std::exception& e, const std::string& file, const std::string& function, const int& line) {
    std::fprintf(stderr, "exception in %s (%s:%d): %s\n", function.c_str(), file.c_str(), line, e.what());
    std::abort();
}
}  // namespace plb
using plb::exHandler;

#include "palabos3D.h"
#include "palabos3D.hh"

using namespace plb;

static void die(const char* m) {
    std::fprintf(stderr, "plb_voxel: %s\n", m);
    std::exit(1);
}

int main(int argc, char** argv) {
    plbInit(&argc, &argv);
    if (argc == 5 && std::strcmp(argv[1], "--stl") == 0) {
        TriangleSet<double> set(argv[2], std::strcmp(argv[3], "dbl") == 0 ? DBL : FLT);
        std::vector<TriangleSet<double>::Triangle> const& t = set.getTriangles();
        FILE* o = std::fopen(argv[4], "wb");
        if (!o) die("cannot open result");
        const int32_t n = (int32_t)t.size();
        std::fwrite("PLBTRI01", 1, 8, o);
        std::fwrite(&n, sizeof(n), 1, o);
        for (int32_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) std::fwrite(&t[i][k][a], sizeof(double), 1, o);
        std::fclose(o);
        return 0;
    }
    if (argc == 8 && std::strcmp(argv[1], "--scale") == 0) {
        TriangleSet<double> set(argv[2], DBL);
        DEFscaledMesh<double> scaled(set, std::atol(argv[3]), std::atol(argv[4]), std::atol(argv[5]),
                                     (plint)std::atol(argv[6]));
        TriangularSurfaceMesh<double> const& mesh = scaled.getMesh();
        FILE* o = std::fopen(argv[7], "wb");
        if (!o) die("cannot open result");
        const int32_t n = (int32_t)mesh.getNumTriangles();
        std::fwrite("PLBTRI01", 1, 8, o);
        std::fwrite(&n, sizeof(n), 1, o);
        for (int32_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) {
                    const double v = mesh.getVertex(i, k)[a];
                    std::fwrite(&v, sizeof(double), 1, o);
                }
        std::fclose(o);
        return 0;
    }
    if (argc != 3) die("usage: plb_voxel <case> <result> | plb_voxel --stl <file> <flt|dbl> <result>");
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) die("cannot open case");
    char magic[8];
    int32_t h[5];
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "PLBVOX01", 8) != 0) die("bad case file");
    if (std::fread(h, sizeof(int32_t), 5, f) != 5) die("bad case header");
    const int nx = h[0], ny = h[1], nz = h[2], border = h[3], ntri = h[4];
    std::vector<double> v((size_t)ntri * 9);
    if (std::fread(v.data(), sizeof(double), v.size(), f) != v.size()) die("truncated triangles");
    std::fclose(f);

    std::vector<typename TriangleSet<double>::Triangle> tris(ntri);
    for (int t = 0; t < ntri; ++t)
        for (int k = 0; k < 3; ++k)
            tris[t][k] = Array<double, 3>(v[9 * t + 3 * k], v[9 * t + 3 * k + 1], v[9 * t + 3 * k + 2]);
    TriangleSet<double> set(tris);
    DEFscaledMesh<double> mesh(set);
    std::auto_ptr<MultiScalarField3D<int> > flags =
        voxelize(mesh.getMesh(), Box3D(0, nx - 1, 0, ny - 1, 0, nz - 1), (plint)border);

    FILE* o = std::fopen(argv[2], "wb");
    if (!o) die("cannot open result");
    std::fwrite("PLBVXR01", 1, 8, o);
    std::fwrite(h, sizeof(int32_t), 3, o);
    std::vector<int32_t> out((size_t)nx * ny * nz);
    for (int x = 0; x < nx; ++x)
        for (int y = 0; y < ny; ++y)
            for (int z = 0; z < nz; ++z) out[((size_t)x * ny + y) * nz + z] = flags->get(x, y, z);
    std::fwrite(out.data(), sizeof(int32_t), out.size(), o);
    std::fclose(o);
    return 0;
}
