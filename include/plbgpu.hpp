// C++ front end of the GB300 D3Q19 lattice library (header only, over the C
// ABI of plbgpu.h).  The names follow the reference's construction and
// analysis calls so that host code reads like a Palabos program:
//
//   plbgpu::Context ctx(0);
//   plbgpu::Lattice3D lattice(ctx, nx, ny, nz, omega);          // MultiBlockLattice3D(nx,ny,nz,new BGKdynamics(omega))
//   lattice.periodicity(true, false, false);                    // lattice.periodicity().toggle(0, true)
//   lattice.defineDynamics(box, PLBGPU_BOUNCEBACK);              // defineDynamics(lattice, box, new BounceBack<T,D>)
//   lattice.addVelocityBoundary(box, 0, -1);                    // bc->addVelocityBoundary0N(box, lattice)
//   lattice.setBoundaryVelocity(box, 0.02, 0., 0.);             // setBoundaryVelocity(lattice, box, u)
//   lattice.initializeAtEquilibrium(lattice.boundingBox(), 1., 0., 0., 0.);
//   lattice.initialize();                                       // lattice.initialize()
//   lattice.collideAndStream();                                 // lattice.collideAndStream()
//   double e = lattice.computeAverageEnergy();                  // computeAverageEnergy(lattice)
//
// Failures of the C ABI are thrown as plbgpu::Error (a std::runtime_error
// carrying the status code and the library's message).
#ifndef PLBGPU_HPP
#define PLBGPU_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "plbgpu.h"

namespace plbgpu {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

// Inclusive box, like plb::Box3D.
struct Box {
    int x0, x1, y0, y1, z0, z1;
    long cells() const { return (long)(x1 - x0 + 1) * (y1 - y0 + 1) * (z1 - z0 + 1); }
};

class Context {
public:
    explicit Context(int device = 0) {
        int rc = plbgpu_create(device, &ctx_);
        if (rc != PLBGPU_OK) throw Error(rc, "plbgpu_create failed for CUDA device " + std::to_string(device));
    }
    ~Context() {
        if (ctx_) plbgpu_destroy(ctx_);
    }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;
    plbgpu_ctx* get() const { return ctx_; }
    void check(int rc) const {
        if (rc != PLBGPU_OK) throw Error(rc, plbgpu_last_error(ctx_));
    }
    void synchronize() const { check(plbgpu_synchronize(ctx_)); }
    unsigned long long launchCount() const {
        unsigned long long n = 0;
        check(plbgpu_launch_count(ctx_, &n));
        return n;
    }

private:
    plbgpu_ctx* ctx_ = nullptr;
};

class Lattice3D {
public:
    Lattice3D(Context& ctx, int nx, int ny, int nz, double omega, int precision = PLBGPU_FP64, double rho0 = 1.0,
              double bbRho = 0.0)
        : ctx_(ctx), nx_(nx), ny_(ny), nz_(nz) {
        ctx_.check(plbgpu_add_domain(ctx_.get(), nx, ny, nz, precision, &h_));
        ctx_.check(plbgpu_set_params(ctx_.get(), h_, omega, rho0, bbRho));
    }
    ~Lattice3D() { plbgpu_remove_domain(ctx_.get(), h_); }
    Lattice3D(const Lattice3D&) = delete;
    Lattice3D& operator=(const Lattice3D&) = delete;

    int handle() const { return h_; }
    Box boundingBox() const { return Box{0, nx_ - 1, 0, ny_ - 1, 0, nz_ - 1}; }

    void periodicity(bool px, bool py, bool pz) {
        ctx_.check(plbgpu_set_periodicity(ctx_.get(), h_, px, py, pz));
    }
    void setParameters(double omega, double rho0 = 1.0, double bbRho = 0.0) {
        ctx_.check(plbgpu_set_params(ctx_.get(), h_, omega, rho0, bbRho));
    }
    void defineDynamics(const Box& b, int kind) {
        ctx_.check(plbgpu_define_dynamics(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, kind));
    }
    void setKinds(const Box& b, const std::vector<uint8_t>& kinds) {
        ctx_.check(plbgpu_set_kinds(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, kinds.data(), kinds.size()));
    }
    // Wrapped regularized (or Zou/He) face conditions: direction 0/1/2, orientation -1/+1.
    void addVelocityBoundary(const Box& b, int direction, int orientation, bool zouHe = false) {
        addBoundary(b, (zouHe ? PLBGPU_ZOUHE_VELOCITY : PLBGPU_REG_VELOCITY) + 2 * direction + (orientation > 0));
    }
    // addExternalVelocityEdge{plane}{N|P}{N|P}: normal1 along (plane+1)%3, normal2 along (plane+2)%3.
    void addExternalVelocityEdge(const Box& b, int plane, int normal1, int normal2) {
        addBoundary(b, PLBGPU_VELOCITY_EDGE + 4 * plane + 2 * (normal1 > 0) + (normal2 > 0));
    }
    // addExternalVelocityCorner{N|P}{N|P}{N|P}(x, y, z, lattice).
    void addExternalVelocityCorner(int x, int y, int z, int xNormal, int yNormal, int zNormal) {
        addBoundary(Box{x, x, y, y, z, z},
                    PLBGPU_VELOCITY_CORNER + 4 * (xNormal > 0) + 2 * (yNormal > 0) + (zNormal > 0));
    }
    // bc->setVelocityConditionOnBlockBoundaries(lattice, box): faces, edges and corners.
    void setVelocityConditionOnBlockBoundaries(const Box& b) {
        ctx_.check(plbgpu_set_velocity_condition_on_block_boundaries(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0,
                                                                      b.z1));
    }
    void setVelocityConditionOnBlockBoundaries() { setVelocityConditionOnBlockBoundaries(boundingBox()); }
    void addPressureBoundary(const Box& b, int direction, int orientation, bool zouHe = false) {
        addBoundary(b, (zouHe ? PLBGPU_ZOUHE_PRESSURE : PLBGPU_REG_PRESSURE) + 2 * direction + (orientation > 0));
    }
    // A face, edge or corner kind plus the data-processor record the
    // reference's boundary instantiator adds with it.
    void addBoundary(const Box& b, int kind) {
        ctx_.check(plbgpu_add_boundary(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, kind));
    }
    // The lattice's data-processor list as saved states describe it.
    int processorCount() const {
        int n = 0;
        ctx_.check(plbgpu_processor_count(ctx_.get(), h_, &n));
        return n;
    }
    void setBoundaryVelocity(const Box& b, double ux, double uy, double uz) {
        ctx_.check(plbgpu_set_boundary_velocity(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, ux, uy, uz));
    }
    void setBoundaryVelocity(const Box& b, const std::vector<double>& u) {
        ctx_.check(plbgpu_set_boundary_velocity_field(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, u.data(),
                                                      u.size()));
    }
    void setBoundaryDensity(const Box& b, double rho) {
        ctx_.check(plbgpu_set_boundary_density(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, rho));
    }
    void setBoundaryDensity(const Box& b, const std::vector<double>& rho) {
        ctx_.check(plbgpu_set_boundary_density_field(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, rho.data(),
                                                     rho.size()));
    }
    void setExternalVector(const Box& b, double fx, double fy, double fz) {
        ctx_.check(plbgpu_set_force(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, fx, fy, fz));
    }
    void setExternalVector(const Box& b, const std::vector<double>& f) {
        ctx_.check(plbgpu_set_force_field(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, f.data(), f.size()));
    }
    void initializeMomentumExchange() { ctx_.check(plbgpu_initialize_momentum_exchange(ctx_.get(), h_)); }
    void initializeAtEquilibrium(const Box& b, double rho, double ux, double uy, double uz) {
        ctx_.check(plbgpu_initialize_at_equilibrium(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, rho, ux, uy,
                                                    uz));
    }
    void initialize() { ctx_.check(plbgpu_initialize(ctx_.get(), h_)); }

    // Populations (FP64 f-bar, [x][y][z][19]) in and out.
    void send(const Box& b, const std::vector<double>& f) {
        ctx_.check(plbgpu_send(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, f.data(), f.size()));
    }
    std::vector<double> receive(const Box& b) const {
        std::vector<double> f((size_t)b.cells() * 19);
        ctx_.check(plbgpu_receive(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, f.data(), f.size()));
        return f;
    }

    void collideAndStream(int steps = 1, bool gatherStatistics = true) {
        ctx_.check(plbgpu_collide_and_stream(ctx_.get(), h_, steps, gatherStatistics));
    }
    // The whole domain's populations f sent, `steps` steps run and the state
    // received back into f, the transfers overlapped with the first and last
    // steps (plbgpu_run_host).  Returns the statistics of every
    // statsEvery-th step and of the last one, 7 values each.
    std::vector<double> runHost(std::vector<double>& f, int steps, int statsEvery = 0) {
        const size_t records = statsEvery > 0 ? (size_t)((steps + statsEvery - 1) / statsEvery) : 0;
        std::vector<double> stats(7 * records);
        ctx_.check(plbgpu_run_host(ctx_.get(), h_, f.data(), f.data(), f.size(), steps, statsEvery, stats.data(),
                                   stats.size()));
        return stats;
    }
    // External rho-bar / j fields and ExternalRhoJcollideAndStream3D steps
    // (values: rho-bar, jx, jy, jz per cell, z fastest).
    void computeRhoBarJ() { ctx_.check(plbgpu_compute_rhobar_j(ctx_.get(), h_)); }
    void setRhoBarJ(const Box& b, const std::vector<double>& values) {
        ctx_.check(plbgpu_set_rhobar_j(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, values.data(),
                                       values.size()));
    }
    std::vector<double> getRhoBarJ(const Box& b) const {
        std::vector<double> v((size_t)b.cells() * 4);
        ctx_.check(plbgpu_get_rhobar_j(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, v.data(), v.size()));
        return v;
    }
    void collideAndStreamExternal(int steps = 1, bool recompute = true, bool gatherStatistics = false) {
        ctx_.check(plbgpu_collide_and_stream_external(ctx_.get(), h_, steps, recompute, gatherStatistics));
    }

    // getInternalStatistics(): average rho-bar, average u^2, max u^2, drag x/y/z, cell count.
    std::vector<double> internalStatistics() const {
        std::vector<double> s(7);
        ctx_.check(plbgpu_get_stats(ctx_.get(), h_, s.data()));
        return s;
    }
    double computeAverageEnergy(const Box& b) const {
        double e, r;
        ctx_.check(plbgpu_reduce(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, &e, &r));
        return e;
    }
    double computeAverageDensity(const Box& b) const {
        double e, r;
        ctx_.check(plbgpu_reduce(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, &e, &r));
        return r;
    }
    double computeAverageEnergy() const { return computeAverageEnergy(boundingBox()); }
    double computeAverageDensity() const { return computeAverageDensity(boundingBox()); }
    std::vector<double> computeVelocity(const Box& b) const {
        std::vector<double> u((size_t)b.cells() * 3);
        ctx_.check(plbgpu_compute_velocity(ctx_.get(), h_, b.x0, b.x1, b.y0, b.y1, b.z0, b.z1, u.data(), u.size()));
        return u;
    }

    // Checkpoints in the reference's formats: saveBinaryBlock / loadBinaryBlock
    // (io/serializerIO_3D.cpp:37-60) and parallelIO::save / load, with or
    // without dynamic content (io/multiBlockWriter3D.cpp:201-213,
    // io/multiBlockReader3D.cpp:261-270).  `what` is a PLBGPU_BLOCK_* kind.
    void saveBinaryBlock(const std::string& path, int what = PLBGPU_BLOCK_LATTICE, bool enforceUint = false) {
        ctx_.check(plbgpu_save_binary_block(ctx_.get(), h_, what, path.c_str(), enforceUint));
    }
    void loadBinaryBlock(const std::string& path, int what = PLBGPU_BLOCK_LATTICE, bool enforceUint = false) {
        ctx_.check(plbgpu_load_binary_block(ctx_.get(), h_, what, path.c_str(), enforceUint));
    }
    void saveState(const std::string& base, bool dynamicContent = true, int what = PLBGPU_BLOCK_LATTICE) {
        ctx_.check(dynamicContent ? plbgpu_save_state_dynamic(ctx_.get(), h_, what, base.c_str())
                                  : plbgpu_save_state(ctx_.get(), h_, what, base.c_str()));
    }
    void loadState(const std::string& plb, bool dynamicContent = true, int what = PLBGPU_BLOCK_LATTICE) {
        ctx_.check(dynamicContent ? plbgpu_load_state_dynamic(ctx_.get(), h_, what, plb.c_str())
                                  : plbgpu_load_state(ctx_.get(), h_, what, plb.c_str()));
    }

private:
    Context& ctx_;
    int nx_, ny_, nz_;
    int h_ = -1;
};

}  // namespace plbgpu

#endif  // PLBGPU_HPP
