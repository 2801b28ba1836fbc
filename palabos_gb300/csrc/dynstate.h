// Dynamic content of parallelIO states: the serialized dynamics chain that
// parallelIO::save(block, base, true) writes in front of every cell's static
// record (atomicBlock/blockLattice3D.hh:703-722 send_all, :812-845
// receive_regenerate), in the layout of HierarchicSerializer
// (core/hierarchicSerializer.h:152-230):
//
//   int numDynamics, then per dynamics of the chain (outermost first):
//     int id, int numValues, then runs of values of one size:
//       int size, int count, count values of `size` bytes
//   (a new run starts when the value size changes or a new dynamics begins).
//
// What each dynamics of the GPU kinds serializes:
//   BGK, BGK_ExternalForce_Guo      omega                  (core/dynamics.hh:119-122)
//   BGK_Incompressible              omega, invRho0
//   BounceBack, NoDynamics          rho                    (core/dynamics.hh:770-773, 955-958)
//   MomentumExchangeBounceBack      rho, int n, n directions (plint), 3 force ids (plint)
//                                                          (boundaryCondition/bounceBackModels.hh:75-84)
//   Boundary_*Velocity_d_o,         u[3], bool automaticPrepareCollision, then the base
//   Boundary_StoreVelocity          dynamics (boundaryDynamics.hh:315-321, core/dynamics.hh:445-450)
//   Boundary_*Density_d_o,          rhoBar, bool, then the base (boundaryDynamics.hh:238-242)
//   Boundary_ZouHePressure_d_o
//
// Host-only C++ (no CUDA), used by the library's state reader and writer;
// tests/cpp/dynstate_check.cpp re-encodes states the reference wrote with it.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "plbgpu.h"

namespace plbgpu_dyn {

// Name of the dynamics class (its registry name) of a GPU kind ("" for none).
inline std::string kindName(int k) {
    static const char* basic[6] = {"BGK", "BGK_ExternalForce_Guo", "BGK_Incompressible", "BounceBack",
                                   "MomentumExchangeBounceBack", "NoDynamics"};
    if (k >= 0 && k < 6) return basic[k];
    if (k >= PLBGPU_REG_VELOCITY && k < PLBGPU_VELOCITY_EDGE) {
        static const char* fam[4] = {"Boundary_RegularizedVelocity", "Boundary_RegularizedDensity",
                                     "Boundary_ZouHeVelocity", "Boundary_ZouHePressure"};
        const int r = k - PLBGPU_REG_VELOCITY, face = r % 6;
        char buf[64];
        snprintf(buf, sizeof(buf), "%s_%d_%d", fam[r / 6], face / 2, face % 2 ? 1 : -1);
        return buf;
    }
    if (k >= PLBGPU_VELOCITY_EDGE && k < PLBGPU_VELOCITY_CORNER + 8) return "Boundary_StoreVelocity";
    return "";
}

inline bool isComposite(int k) { return k >= PLBGPU_REG_VELOCITY && k < PLBGPU_VELOCITY_CORNER + 8; }
inline bool isDensityKind(int k) {
    return (k >= PLBGPU_REG_PRESSURE && k < PLBGPU_ZOUHE_VELOCITY) ||
           (k >= PLBGPU_ZOUHE_PRESSURE && k < PLBGPU_VELOCITY_EDGE);
}

// Registry ids this library writes (any ids are valid: the state's
// DynamicsDict maps them to names, io/multiBlockWriter3D.cpp:92-110).
inline int kindId(int k) { return k >= PLBGPU_VELOCITY_EDGE ? 31 : k + 1; }
constexpr int kBgkId = 1;

// HierarchicSerializer's byte layout.
class ChainWriter {
public:
    ChainWriter(std::vector<char>& out, int topId) : out_(out) {
        numDynPos_ = slot();
        next(topId);
    }
    void next(int id) {
        put<int32_t>(id);
        numValPos_ = slot();
        runSize_ = 0;
        bump(numDynPos_);
    }
    template <typename T> void value(T v) {
        if ((int)sizeof(T) != runSize_) {
            runSize_ = (int)sizeof(T);
            put<int32_t>(runSize_);
            runPos_ = slot();
        }
        put<T>(v);
        bump(runPos_);
        bump(numValPos_);
    }

private:
    template <typename T> void put(T v) {
        const size_t p = out_.size();
        out_.resize(p + sizeof(T));
        memcpy(&out_[p], &v, sizeof(T));
    }
    size_t slot() {
        const size_t p = out_.size();
        put<int32_t>(0);
        return p;
    }
    void bump(size_t p) {
        int32_t v;
        memcpy(&v, &out_[p], 4);
        ++v;
        memcpy(&out_[p], &v, 4);
    }
    std::vector<char>& out_;
    size_t numDynPos_ = 0, numValPos_ = 0, runPos_ = 0;
    int runSize_ = 0;
};

// Domain-wide parameters of the GPU lattice.
struct Params {
    double omega = 1.0, rho0 = 1.0, bbRho = 0.0;
};

// Kind byte of a cell outside the lattice of a sparse domain.
constexpr int kOutside = 255;

// Append the dynamics chain of one cell of kind k.  bc: the cell's three
// boundary values (velocity, or density in bc[0]); mask: its momentum-exchange
// fluid directions (bit i for direction i).  A cell outside the lattice is
// written as NoDynamics (its populations are zero): a reference lattice built
// on the same sparse blocks has no cell there and ignores it on loading.
// ids: the registry ids to write by dynamics name (default: kindId / kBgkId).
inline void appendCell(std::vector<char>& out, int k, const double* bc, uint32_t mask, const Params& p,
                       const std::map<std::string, int>* ids = nullptr) {
    if (k == kOutside) k = PLBGPU_NODYNAMICS;
    auto idOf = [ids](const std::string& name, int dflt) {
        if (ids) {
            auto it = ids->find(name);
            if (it != ids->end()) return it->second;
        }
        return dflt;
    };
    ChainWriter w(out, idOf(kindName(k), kindId(k)));
    if (k == PLBGPU_BGK || k == PLBGPU_GUO) {
        w.value(p.omega);
    } else if (k == PLBGPU_INCBGK) {
        w.value(p.omega);
        w.value((double)1 / p.rho0);
    } else if (k == PLBGPU_BOUNCEBACK || k == PLBGPU_NODYNAMICS) {
        w.value(p.bbRho);
    } else if (k == PLBGPU_MOMENTUM_EXCHANGE) {
        w.value(p.bbRho);
        int32_t n = 0;
        for (int i = 0; i < 19; ++i) n += (mask >> i) & 1u;
        w.value(n);
        for (int i = 0; i < 19; ++i)
            if ((mask >> i) & 1u) w.value((int64_t)i);
        for (int64_t a = 0; a < 3; ++a) w.value(a);   // the first three subscribed sums: the drag
    } else {   // composite: stored value, automaticPrepareCollision, then the BGK base
        if (isDensityKind(k)) {
            w.value(bc[0] - 1.0);   // rhoToRhoBar, as setBoundaryDensity stores it
        } else {
            w.value(bc[0]);
            w.value(bc[1]);
            w.value(bc[2]);
        }
        w.value((bool)(k >= PLBGPU_VELOCITY_EDGE));   // edges and corners prepare themselves
        w.next(idOf("BGK", kBgkId));
        w.value(p.omega);
    }
}

// ------------------------------------------------------------ reading

// One cell's decoded dynamics.
struct Cell {
    int kind = -1;
    double bc[3] = {0, 0, 0};
    uint32_t mask = 0;
    bool hasOmega = false, hasInvRho0 = false, hasRho = false;
    double omega = 0, invRho0 = 0, rho = 0;
};

// Values of one dynamics in serialization order, with their byte sizes.
struct Values {
    std::vector<std::pair<int, const char*>> v;
    size_t i = 0;
    template <typename T> bool get(T& out) {
        if (i >= v.size() || v[i].first != (int)sizeof(T)) return false;
        memcpy(&out, v[i].second, sizeof(T));
        ++i;
        return true;
    }
    bool done() const { return i == v.size(); }
};

inline bool readInt(const char* p, size_t avail, size_t& pos, int32_t& out) {
    if (pos + 4 > avail) return false;
    memcpy(&out, p + pos, 4);
    pos += 4;
    return true;
}

// Edge or corner kind of a stored-velocity cell from its place on the lattice box.
inline int surfaceKind(int x, int y, int z, int nx, int ny, int nz) {
    const int q[3] = {x, y, z}, n[3] = {nx, ny, nz};
    int side[3], count = 0;
    for (int a = 0; a < 3; ++a) {
        side[a] = q[a] == 0 ? -1 : (q[a] == n[a] - 1 ? 1 : 0);
        count += side[a] != 0;
    }
    if (count == 3) return PLBGPU_VELOCITY_CORNER + 4 * (side[0] > 0) + 2 * (side[1] > 0) + (side[2] > 0);
    if (count == 2) {
        const int plane = !side[0] ? 0 : (!side[1] ? 1 : 2);
        return PLBGPU_VELOCITY_EDGE + 4 * plane + 2 * (side[(plane + 1) % 3] > 0) + (side[(plane + 2) % 3] > 0);
    }
    return -1;
}

// Kind of a (non-stored-velocity) dynamics name; -1 when the GPU has none.
inline int kindOfName(const std::string& name) {
    for (int k = 0; k < PLBGPU_VELOCITY_EDGE; ++k)
        if (kindName(k) == name) return k;
    return -1;
}

// Decode the dynamics chain at p[pos..avail) of the cell at (x, y, z) of an
// nx*ny*nz lattice; names maps the state's ids to dynamics names.  Returns ""
// on success (pos is then past the chain), else what is wrong.
inline std::string readCell(const char* p, size_t avail, size_t& pos, const std::map<int, std::string>& names,
                            int x, int y, int z, int nx, int ny, int nz, Cell& c) {
    int32_t nd;
    if (!readInt(p, avail, pos, nd) || nd < 1 || nd > 8) return "bad dynamics chain";
    std::vector<std::string> chain(nd);
    std::vector<Values> vals(nd);
    for (int d = 0; d < nd; ++d) {
        int32_t id, nv;
        if (!readInt(p, avail, pos, id) || !readInt(p, avail, pos, nv) || nv < 0) return "bad dynamics chain";
        auto it = names.find(id);
        if (it == names.end()) return "dynamics id " + std::to_string(id) + " is not in the DynamicsDict";
        chain[d] = it->second;
        int32_t got = 0;
        while (got < nv) {
            int32_t size, count;
            if (!readInt(p, avail, pos, size) || !readInt(p, avail, pos, count) || size < 1 || size > 16 ||
                count < 1 || count > nv - got)
                return "bad value run in the chain of " + chain[d];
            if (pos + (size_t)size * count > avail) return "truncated dynamics data";
            for (int32_t r = 0; r < count; ++r) vals[d].v.push_back({size, p + pos + (size_t)r * size});
            pos += (size_t)size * count;
            got += count;
        }
    }
    const std::string& top = chain[0];
    Values& v = vals[0];
    const std::string bad = "unexpected values in the serialization of " + top;
    if (top == "Boundary_StoreVelocity" || kindOfName(top) >= PLBGPU_REG_VELOCITY) {
        c.kind = top == "Boundary_StoreVelocity" ? surfaceKind(x, y, z, nx, ny, nz) : kindOfName(top);
        if (c.kind < 0) return "a stored-velocity cell that is not on an edge or corner of the lattice";
        if (isDensityKind(c.kind)) {
            double rhoBar;
            if (!v.get(rhoBar)) return bad;
            c.bc[0] = rhoBar + 1.0;   // the density setBoundaryDensity would be given
        } else {
            for (int a = 0; a < 3; ++a)
                if (!v.get(c.bc[a])) return bad;
        }
        bool prep;
        if (!v.get(prep) || !v.done()) return bad;
        if (nd != 2 || chain[1] != "BGK") return top + " around '" + (nd > 1 ? chain[1] : "") + "' has no GPU kind";
        if (!vals[1].get(c.omega) || !vals[1].done()) return "unexpected values in the serialization of BGK";
        c.hasOmega = true;
        return "";
    }
    if (nd != 1) return "composite dynamics '" + top + "' has no GPU kind";
    c.kind = kindOfName(top);
    if (c.kind < 0) return "dynamics '" + top + "' has no GPU kind";
    switch (c.kind) {
    case PLBGPU_BGK:
    case PLBGPU_GUO:
        if (!v.get(c.omega) || !v.done()) return bad;
        c.hasOmega = true;
        break;
    case PLBGPU_INCBGK:
        if (!v.get(c.omega) || !v.get(c.invRho0) || !v.done()) return bad;
        c.hasOmega = c.hasInvRho0 = true;
        break;
    case PLBGPU_BOUNCEBACK:
    case PLBGPU_NODYNAMICS:
        if (!v.get(c.rho) || !v.done()) return bad;
        c.hasRho = true;
        break;
    default: {   // momentum exchange
        int32_t n;
        if (!v.get(c.rho) || !v.get(n) || n < 0 || n > 19) return bad;
        c.hasRho = true;
        for (int32_t i = 0; i < n; ++i) {
            int64_t dir;
            if (!v.get(dir) || dir < 0 || dir > 18) return bad;
            c.mask |= 1u << dir;
        }
        for (int a = 0; a < 3; ++a) {
            int64_t fid;
            if (!v.get(fid)) return bad;
        }
        if (!v.done()) return bad;
    }
    }
    return "";
}

// rho0 whose reciprocal (as the library computes it, 1/rho0) is invRho0;
// false when no double has that reciprocal.
inline bool rho0FromInverse(double invRho0, double& rho0) {
    double c[5];
    c[0] = (double)1 / invRho0;
    c[1] = std::nextafter(c[0], INFINITY);
    c[2] = std::nextafter(c[0], -INFINITY);
    c[3] = std::nextafter(c[1], INFINITY);
    c[4] = std::nextafter(c[2], -INFINITY);
    for (double r : c)
        if ((double)1 / r == invRho0) {
            rho0 = r;
            return true;
        }
    return false;
}

}  // namespace plbgpu_dyn
