// CPU stand-in for the co-processor calls of libplbgpu (include/plbgpu.h,
// "co-processor form"), built on the oracle -- the reference's arithmetic
// restated in C (oracle/plb_oracle.c).  TEST INFRASTRUCTURE: it lets the
// Palabos adapter (include/plbgpu_coprocessor3d.hh) run end to end through the
// reference's own co-processor wiring on a machine without a GPU.  The GPU
// library's co-processor calls are checked against the same oracle on the GPU
// (tests/test_gpu_parity.py), so the two checks together pin the adapter on
// the GPU to the reference's co-processor path.
//
// A domain is a non-periodic all-BGK block, as the reference's example
// co-processor builds it (coProcessors/coProcessor3D.hh:36-46); the FP32 calls
// keep the same FP64 state and convert the records.
#include <cstdint>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "plbgpu.h"

extern "C" {
typedef struct {
    int nx, ny, nz;
    int periodic[3];
    double omega, rho0, bbRho;
} orc_params;
int orc_run(const orc_params* p, const uint8_t* flags, const double* bcval, const double* force, double* f,
            int nsteps, double* stats);
}

namespace {
struct FakeDomain {
    orc_params p;
    std::vector<uint8_t> flags;
    std::vector<double> f;
};
}  // namespace

struct plbgpu_ctx {
    std::map<int, FakeDomain> domains;
    int next = 0;
};

namespace {

FakeDomain* find(plbgpu_ctx* c, int h) {
    if (!c) return nullptr;
    auto it = c->domains.find(h);
    return it == c->domains.end() ? nullptr : &it->second;
}

int addDomain(plbgpu_ctx* c, long nx, long ny, long nz, double omega, int* handle) {
    if (!c || !handle || nx < 1 || ny < 1 || nz < 1) return 0;
    FakeDomain d;
    d.p.nx = (int)nx; d.p.ny = (int)ny; d.p.nz = (int)nz;
    d.p.periodic[0] = d.p.periodic[1] = d.p.periodic[2] = 0;
    d.p.omega = omega; d.p.rho0 = 1.0; d.p.bbRho = 0.0;
    d.flags.assign((size_t)(nx * ny * nz), 0);           // BGK
    d.f.assign((size_t)(nx * ny * nz) * 19, 0.0);
    *handle = c->next++;
    c->domains[*handle] = d;
    return 1;
}

// Copy the records of a sub-box between the caller's buffer (T) and the state.
template <typename T>
int transfer(plbgpu_ctx* c, int h, long x0, long x1, long y0, long y1, long z0, long z1, T* data, size_t nbytes,
             bool toDomain) {
    FakeDomain* d = find(c, h);
    if (!d || x0 < 0 || y0 < 0 || z0 < 0 || x1 >= d->p.nx || y1 >= d->p.ny || z1 >= d->p.nz || x0 > x1 ||
        y0 > y1 || z0 > z1)
        return 0;
    const size_t cells = (size_t)(x1 - x0 + 1) * (y1 - y0 + 1) * (z1 - z0 + 1);
    if (nbytes != cells * 19 * sizeof(T)) return 0;
    size_t o = 0;
    for (long x = x0; x <= x1; ++x)
        for (long y = y0; y <= y1; ++y)
            for (long z = z0; z <= z1; ++z, o += 19) {
                double* f = d->f.data() + (((size_t)x * d->p.ny + y) * d->p.nz + z) * 19;
                for (int i = 0; i < 19; ++i) {
                    if (toDomain) f[i] = (double)data[o + i];
                    else data[o + i] = (T)f[i];
                }
            }
    return 1;
}

}  // namespace

extern "C" {

int plbgpu_create(int, plbgpu_ctx** out) {
    if (!out) return PLBGPU_ERR_ARG;
    *out = new (std::nothrow) plbgpu_ctx();
    return *out ? PLBGPU_OK : PLBGPU_ERR_NOMEM;
}
int plbgpu_destroy(plbgpu_ctx* c) {
    delete c;
    return PLBGPU_OK;
}
int plbgpu_cp_add_domain(plbgpu_ctx* c, long nx, long ny, long nz, double omega, int* handle) {
    return addDomain(c, nx, ny, nz, omega, handle);
}
int plbgpu_cp_add_domain_f32(plbgpu_ctx* c, long nx, long ny, long nz, double omega, int* handle) {
    return addDomain(c, nx, ny, nz, omega, handle);
}
int plbgpu_cp_send(plbgpu_ctx* c, int h, long x0, long x1, long y0, long y1, long z0, long z1, const char* data,
                   size_t nbytes) {
    return transfer<double>(c, h, x0, x1, y0, y1, z0, z1, (double*)data, nbytes, true);
}
int plbgpu_cp_receive(plbgpu_ctx* c, int h, long x0, long x1, long y0, long y1, long z0, long z1, char* data,
                      size_t nbytes) {
    return transfer<double>(c, h, x0, x1, y0, y1, z0, z1, (double*)data, nbytes, false);
}
int plbgpu_cp_send_f32(plbgpu_ctx* c, int h, long x0, long x1, long y0, long y1, long z0, long z1,
                       const char* data, size_t nbytes) {
    return transfer<float>(c, h, x0, x1, y0, y1, z0, z1, (float*)data, nbytes, true);
}
int plbgpu_cp_receive_f32(plbgpu_ctx* c, int h, long x0, long x1, long y0, long y1, long z0, long z1, char* data,
                          size_t nbytes) {
    return transfer<float>(c, h, x0, x1, y0, y1, z0, z1, (float*)data, nbytes, false);
}
int plbgpu_cp_collide_and_stream(plbgpu_ctx* c, int h) {
    FakeDomain* d = find(c, h);
    if (!d) return 0;
    double none[3] = {0., 0., 0.};
    return orc_run(&d->p, d->flags.data(), none, none, d->f.data(), 1, nullptr) == 0 ? 1 : 0;
}

}  // extern "C"
