// Palabos co-processor adapter: plb::CoProcessor3D<T> implemented on the GB300
// library.  Include it after the Palabos headers (it names plb::CoProcessor3D,
// plb::Box3D and plb::plint) and register an instance as the default
// co-processor; initiateCoProcessors / transferToCoProcessors /
// MultiBlockLattice3D::collideAndStream / transferFromCoProcessors then run
// every pure-BGK block on the GPU unchanged
// (coProcessors/coProcessorCommunication3D.hh:34-125,
//  multiBlock/multiBlockLattice3D.hh:318-357).
//
// The four calls keep the reference's contract (coProcessors/coProcessor3D.h:41-116):
// a domain is a non-periodic BGK block addressed 0..n-1 with the given omega;
// data is std::vector<char> holding 19 T per cell, z fastest; receive() resizes
// the vector; collideAndStream() blocks; every call returns 1 on success and 0
// on failure.  T = double runs the FP64 form (bit-identical to the reference's
// own example co-processor, D3Q19ExampleCoProcessor3D); T = float runs the
// FP32 form (FP32 arithmetic and storage, 19 floats per cell).
#ifndef PLBGPU_COPROCESSOR3D_HH
#define PLBGPU_COPROCESSOR3D_HH

#include <vector>

#include "plbgpu.h"

namespace plbgpu {

// The C calls of each precision, picked by overload on the lattice type.
namespace cp {
inline int addDomain(plbgpu_ctx* c, long nx, long ny, long nz, double omega, int* h, double) {
    return plbgpu_cp_add_domain(c, nx, ny, nz, omega, h);
}
inline int addDomain(plbgpu_ctx* c, long nx, long ny, long nz, double omega, int* h, float) {
    return plbgpu_cp_add_domain_f32(c, nx, ny, nz, omega, h);
}
inline int send(plbgpu_ctx* c, int h, const plb::Box3D& d, const char* data, size_t n, double) {
    return plbgpu_cp_send(c, h, (long)d.x0, (long)d.x1, (long)d.y0, (long)d.y1, (long)d.z0, (long)d.z1, data, n);
}
inline int send(plbgpu_ctx* c, int h, const plb::Box3D& d, const char* data, size_t n, float) {
    return plbgpu_cp_send_f32(c, h, (long)d.x0, (long)d.x1, (long)d.y0, (long)d.y1, (long)d.z0, (long)d.z1, data, n);
}
inline int receive(plbgpu_ctx* c, int h, const plb::Box3D& d, char* data, size_t n, double) {
    return plbgpu_cp_receive(c, h, (long)d.x0, (long)d.x1, (long)d.y0, (long)d.y1, (long)d.z0, (long)d.z1, data, n);
}
inline int receive(plbgpu_ctx* c, int h, const plb::Box3D& d, char* data, size_t n, float) {
    return plbgpu_cp_receive_f32(c, h, (long)d.x0, (long)d.x1, (long)d.y0, (long)d.y1, (long)d.z0, (long)d.z1, data,
                                 n);
}
}  // namespace cp

template <typename T>
class GpuD3Q19CoProcessor3D : public plb::CoProcessor3D<T> {
public:
    explicit GpuD3Q19CoProcessor3D(int device = 0) {
        if (plbgpu_create(device, &ctx_) != PLBGPU_OK) ctx_ = nullptr;
    }
    virtual ~GpuD3Q19CoProcessor3D() {
        if (ctx_) plbgpu_destroy(ctx_);
    }
    virtual int addDomain(plb::plint nx, plb::plint ny, plb::plint nz, T omega, int& domainHandle) {
        if (!ctx_) return 0;
        return cp::addDomain(ctx_, (long)nx, (long)ny, (long)nz, (double)omega, &domainHandle, T());
    }
    virtual int send(int domainHandle, plb::Box3D const& d, std::vector<char> const& data) {
        if (!ctx_) return 0;
        return cp::send(ctx_, domainHandle, d, data.data(), data.size(), T());
    }
    virtual int receive(int domainHandle, plb::Box3D const& d, std::vector<char>& data) const {
        if (!ctx_) return 0;
        data.resize((size_t)d.nCells() * 19 * sizeof(T));
        return cp::receive(ctx_, domainHandle, d, data.data(), data.size(), T());
    }
    virtual int collideAndStream(int domainHandle) {
        if (!ctx_) return 0;
        return plbgpu_cp_collide_and_stream(ctx_, domainHandle);
    }
    plbgpu_ctx* context() const { return ctx_; }

private:
    plbgpu_ctx* ctx_ = nullptr;
};

}  // namespace plbgpu

#endif  // PLBGPU_COPROCESSOR3D_HH
