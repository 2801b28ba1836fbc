/*
 * CPU ORACLE -- test infrastructure, not product code.
 *
 * A plain-C restatement of the reference's D3Q19 collide-and-stream step
 * (Palabos MultiBlockLattice3D<double,D3Q19>::collideAndStream with BGK,
 * incompressible BGK, Guo-forced BGK, bounce-back, momentum-exchange
 * bounce-back, no-dynamics, and the wrapped regularized / Zou-He velocity and
 * pressure faces), plus the reductions computeAverageEnergy /
 * computeAverageDensity and the per-step internal statistics.
 *
 * Only the tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
 * may load this library, and only as the checker / the timed CPU baseline.
 * The CUDA library never links it.
 *
 * Parity is pinned: tests/test_oracle_golden.py compares this file's results
 * with golden vectors produced by the unmodified reference (built from its
 * sources by oracle/Makefile.ref, driven by oracle/ref_drivers/plb_case.cpp).
 *
 * Every arithmetic expression keeps the reference's operand order so the
 * results are bit-identical under -ffp-contract=off.  Citations are to files
 * inside the reference's src/ directory.
 *
 * Data layout: f-bar (= f - t_i, roundOffPolicy.h:40-52, 73-89) in canonical
 * order [x][y][z][19], z fastest, exactly the co-processor transfer layout
 * (coProcessors/coProcessor3D.h:84-91).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum {
    K_BGK = 0, K_GUO = 1, K_INCBGK = 2, K_BB = 3, K_MEBB = 4, K_NODYN = 5,
    K_REGVEL = 6, K_REGPRESS = 12, K_ZHVEL = 18, K_ZHPRESS = 24,
    K_EDGE = 30,    /* 30..41: 30 + 4*plane + 2*(normal1>0) + (normal2>0) */
    K_CORNER = 42,  /* 42..49: 42 + 4*(xNormal>0) + 2*(yNormal>0) + (zNormal>0) */
    K_NKINDS = 50,
    K_NONE = 255    /* not part of the lattice: outside every kept block of a sparse domain */
};

/* latticeBoltzmann/nearestNeighborLattices3D.hh:168-180 */
static const int C[19][3] = {
    {0, 0, 0},
    {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {-1, -1, 0}, {-1, 1, 0}, {-1, 0, -1},
    {-1, 0, 1}, {0, -1, -1}, {0, -1, 1},
    {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, -1, 0}, {1, 0, 1},
    {1, 0, -1}, {0, 1, 1}, {0, 1, -1}};

static double T_W[19];
static double CS2, INVCS2;

static void init_constants(void) {
    /* (T)1/(T)3 etc. as in nearestNeighborLattices3D.hh:183-205 */
    T_W[0] = (double)1 / (double)3;
    for (int i = 1; i < 19; ++i) {
        int n2 = C[i][0] * C[i][0] + C[i][1] * C[i][1] + C[i][2] * C[i][2];
        T_W[i] = (n2 == 1) ? (double)1 / (double)18 : (double)1 / (double)36;
    }
    CS2 = (double)1 / (double)3;
    INVCS2 = (double)3;
}

static inline int opp(int i) { return i == 0 ? 0 : (i <= 9 ? i + 9 : i - 9); }

typedef struct {
    int nx, ny, nz;
    int periodic[3];
    double omega, rho0, bbRho;
    const uint8_t* flags;
    const double* bcval; /* N*3 */
    const double* force; /* N*3 (Guo cells) */
    uint32_t* mebbMask;  /* N, bit i = fluid direction i (MEBB cells only) */
    int hasEdges;        /* any edge or corner cell */
    int hasNone;         /* any cell outside the lattice (sparse domain) */
} orc_lattice;

/* ------------------------------------------------------------ moments */

/* momentTemplates3D.h:351-365, 411-425 */
static void get_rhoBar_j(const double* f, double* rhoBar, double j[3]) {
    double surfX_M1 = f[1] + f[4] + f[5] + f[6] + f[7];
    double surfX_P1 = f[10] + f[13] + f[14] + f[15] + f[16];
    double surfY_M1 = f[2] + f[4] + f[8] + f[9] + f[14];
    double surfY_P1 = f[5] + f[11] + f[13] + f[17] + f[18];
    double surfZ_M1 = f[3] + f[6] + f[8] + f[16] + f[18];
    double surfZ_P1 = f[7] + f[9] + f[12] + f[15] + f[17];
    double surfX_0 = f[0] + f[2] + f[3] + f[8] + f[9] + f[11] + f[12] + f[17] + f[18];
    *rhoBar = surfX_M1 + surfX_0 + surfX_P1;
    j[0] = (surfX_P1 - surfX_M1);
    j[1] = (surfY_P1 - surfY_M1);
    j[2] = (surfZ_P1 - surfZ_M1);
}

/* momentTemplates3D.h:372-379 */
static double get_rhoBar(const double* f) {
    double r = f[0];
    for (int i = 1; i < 19; ++i) r = r + f[i];
    return r;
}

/* momentTemplates3D.h:381-396 */
static void get_j(const double* f, double j[3]) {
    double r;
    get_rhoBar_j(f, &r, j);
}

/* dynamicsTemplates3D.h:1994-1997: c.j keeps the reference's left-to-right sum. */
static inline double c_dot(int i, const double j[3]) {
    return (double)C[i][0] * j[0] + (double)C[i][1] * j[1] + (double)C[i][2] * j[2];
}

static inline double bgk_eq(int i, double rhoBar, double invRho, const double j[3], double jSqr) {
    double cj = c_dot(i, j);
    return T_W[i] * (rhoBar + (double)3. * cj + invRho * ((double)4.5 * cj * cj - (double)1.5 * jSqr));
}

static inline double invRhoOf(double rhoBar) { return (double)1 / (rhoBar + (double)1); }

/* ------------------------------------------------------------ collisions */

/* dynamicsTemplates3D.h:2289-2366 */
static double bgk_collision_base(double* f, double rhoBar, const double j[3], double omega, double invRho) {
    double one_m_omega = (double)1 - omega;
    double t0_omega = T_W[0] * omega;
    double t1_omega = T_W[1] * omega;
    double t4_omega = T_W[4] * omega;
    double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    double kx = (double)3 * j[0];
    double ky = (double)3 * j[1];
    double kz = (double)3 * j[2];
    double kxSqr_ = invRho / (double)2 * kx * kx;
    double kySqr_ = invRho / (double)2 * ky * ky;
    double kzSqr_ = invRho / (double)2 * kz * kz;
    double kxky_ = invRho * kx * ky;
    double kxkz_ = invRho * kx * kz;
    double kykz_ = invRho * ky * kz;
    double C1 = rhoBar + invRho * (double)3 * jSqr;
    double C2, C3;

    C3 = -kxSqr_ - kySqr_ - kzSqr_;
    f[0] *= one_m_omega; f[0] += t0_omega * (C1 + C3);

    C2 = -kx; C3 = -kySqr_ - kzSqr_;
    f[1] *= one_m_omega; f[1] += t1_omega * (C1 + C2 + C3);
    f[10] *= one_m_omega; f[10] += t1_omega * (C1 - C2 + C3);

    C2 = -ky; C3 = -kxSqr_ - kzSqr_;
    f[2] *= one_m_omega; f[2] += t1_omega * (C1 + C2 + C3);
    f[11] *= one_m_omega; f[11] += t1_omega * (C1 - C2 + C3);

    C2 = -kz; C3 = -kxSqr_ - kySqr_;
    f[3] *= one_m_omega; f[3] += t1_omega * (C1 + C2 + C3);
    f[12] *= one_m_omega; f[12] += t1_omega * (C1 - C2 + C3);

    C2 = -kx - ky; C3 = kxky_ - kzSqr_;
    f[4] *= one_m_omega; f[4] += t4_omega * (C1 + C2 + C3);
    f[13] *= one_m_omega; f[13] += t4_omega * (C1 - C2 + C3);

    C2 = -kx + ky; C3 = -kxky_ - kzSqr_;
    f[5] *= one_m_omega; f[5] += t4_omega * (C1 + C2 + C3);
    f[14] *= one_m_omega; f[14] += t4_omega * (C1 - C2 + C3);

    C2 = -kx - kz; C3 = kxkz_ - kySqr_;
    f[6] *= one_m_omega; f[6] += t4_omega * (C1 + C2 + C3);
    f[15] *= one_m_omega; f[15] += t4_omega * (C1 - C2 + C3);

    C2 = -kx + kz; C3 = -kxkz_ - kySqr_;
    f[7] *= one_m_omega; f[7] += t4_omega * (C1 + C2 + C3);
    f[16] *= one_m_omega; f[16] += t4_omega * (C1 - C2 + C3);

    C2 = -ky - kz; C3 = kykz_ - kxSqr_;
    f[8] *= one_m_omega; f[8] += t4_omega * (C1 + C2 + C3);
    f[17] *= one_m_omega; f[17] += t4_omega * (C1 - C2 + C3);

    C2 = -ky + kz; C3 = -kykz_ - kxSqr_;
    f[9] *= one_m_omega; f[9] += t4_omega * (C1 + C2 + C3);
    f[18] *= one_m_omega; f[18] += t4_omega * (C1 - C2 + C3);

    return invRho * invRho * jSqr;
}

/* externalForceTemplates3D.h:73-150 (ForcedD3Q19, amplitude 1) */
static void add_guo_force(double* f, const double* F, const double u[3], double omega) {
    double mu = (double)1 * ((double)1 - omega / (double)2);
    const double oneOver6 = (double)1 / (double)6;
    const double oneOver12 = (double)1 / (double)12;
    f[0] += -mu * (F[0] * u[0] + F[1] * u[1] + F[2] * u[2]);
    f[1] += oneOver6 * mu * (F[0] * (-(double)1 + 2 * u[0]) - F[1] * u[1] - F[2] * u[2]);
    f[2] += -oneOver6 * mu * (F[0] * u[0] + F[1] * ((double)1 - 2 * u[1]) + F[2] * u[2]);
    f[3] += -oneOver6 * mu * (F[0] * u[0] + F[1] * u[1] + F[2] * ((double)1 - 2 * u[2]));
    f[4] += oneOver12 * mu * (F[0] * (-(double)1 + 2 * u[0] + 3 * u[1])
                              + F[1] * (-(double)1 + 2 * u[1] + 3 * u[0]) - F[2] * u[2]);
    f[5] += oneOver12 * mu * (F[0] * (-(double)1 + 2 * u[0] - 3 * u[1])
                              + F[1] * ((double)1 + 2 * u[1] - 3 * u[0]) - F[2] * u[2]);
    f[6] += oneOver12 * mu * (F[0] * (-(double)1 + 2 * u[0] + 3 * u[2]) - F[1] * u[1]
                              + F[2] * (-(double)1 + 2 * u[2] + 3 * u[0]));
    f[7] += oneOver12 * mu * (F[0] * (-(double)1 + 2 * u[0] - 3 * u[2]) - F[1] * u[1]
                              + F[2] * ((double)1 + 2 * u[2] - 3 * u[0]));
    f[8] += -oneOver12 * mu * (F[0] * u[0] + F[1] * ((double)1 - 2 * u[1] - 3 * u[2])
                               + F[2] * ((double)1 - 2 * u[2] - 3 * u[1]));
    f[9] += -oneOver12 * mu * (F[0] * u[0] + F[1] * ((double)1 - 2 * u[1] + 3 * u[2])
                               + F[2] * (-(double)1 - 2 * u[2] + 3 * u[1]));
    f[10] += oneOver6 * mu * (F[0] * ((double)1 + 2 * u[0]) - F[1] * u[1] - F[2] * u[2]);
    f[11] += -oneOver6 * mu * (F[0] * u[0] + F[1] * (-(double)1 - 2 * u[1]) + F[2] * u[2]);
    f[12] += -oneOver6 * mu * (F[0] * u[0] + F[1] * u[1] + F[2] * (-(double)1 - 2 * u[2]));
    f[13] += oneOver12 * mu * (F[0] * ((double)1 + 2 * u[0] + 3 * u[1])
                               + F[1] * ((double)1 + 2 * u[1] + 3 * u[0]) - F[2] * u[2]);
    f[14] += oneOver12 * mu * (F[0] * ((double)1 + 2 * u[0] - 3 * u[1])
                               + F[1] * (-(double)1 + 2 * u[1] - 3 * u[0]) - F[2] * u[2]);
    f[15] += oneOver12 * mu * (F[0] * ((double)1 + 2 * u[0] + 3 * u[2]) - F[1] * u[1]
                               + F[2] * ((double)1 + 2 * u[2] + 3 * u[0]));
    f[16] += oneOver12 * mu * (F[0] * ((double)1 + 2 * u[0] - 3 * u[2]) - F[1] * u[1]
                               + F[2] * (-(double)1 + 2 * u[2] - 3 * u[0]));
    f[17] += -oneOver12 * mu * (F[0] * u[0] + F[1] * (-(double)1 - 2 * u[1] - 3 * u[2])
                                + F[2] * (-(double)1 - 2 * u[2] - 3 * u[1]));
    f[18] += -oneOver12 * mu * (F[0] * u[0] + F[1] * (-(double)1 - 2 * u[1] + 3 * u[2])
                                + F[2] * ((double)1 - 2 * u[2] + 3 * u[1]));
}

typedef struct {
    double sumRhoBar, sumUSqr, maxUSqr;
    long count;
    double drag[3];
} orc_stats;

static void swap_halves(double* f) {
    for (int i = 1; i <= 9; ++i) {
        double t = f[i]; f[i] = f[i + 9]; f[i + 9] = t;
    }
}

/* One cell's collision.  isoThermalDynamics.hh:319-330 (BGK), :1408-1419
 * (IncBGK), externalForceDynamics.hh:215-234 (Guo), core/dynamics.hh:783-790
 * (BounceBack), bounceBackModels.hh:100-136 (momentum exchange),
 * core/dynamics.hh:968-971 (NoDynamics).  Boundary-face cells are composite
 * dynamics whose collide() is the base BGK collide (automaticPrepareCollision
 * is false for the wrapped managers, boundaryCondition3D.hh:825-846). */
static void collide_cell(const orc_lattice* L, long id, double* f, orc_stats* st) {
    int k = L->flags[id];
    double rhoBar, j[3], uSqr;
    switch (k) {
    case K_BB:
        swap_halves(f);
        return;
    case K_NODYN: case K_NONE:
        return;
    case K_MEBB: {
        double mom[3] = {0., 0., 0.};
        uint32_t mask = L->mebbMask[id];
        for (int i = 1; i < 19; ++i) {
            if (!(mask & (1u << i))) continue;
            int io = opp(i);
            for (int d = 0; d < 3; ++d) mom[d] += (double)2 * C[i][d] * f[io];
        }
        for (int d = 0; d < 3; ++d) st->drag[d] += -mom[d];
        swap_halves(f);
        return;
    }
    case K_GUO: {
        const double* F = L->force + 3 * id;
        double rb = get_rhoBar(f);
        double rb2, jj[3], u[3];
        get_rhoBar_j(f, &rb2, jj);
        double invRho = invRhoOf(rb2);
        for (int d = 0; d < 3; ++d) u[d] = jj[d] * invRho + F[d] / (double)2;
        double rho = rb + (double)1;
        for (int d = 0; d < 3; ++d) j[d] = rho * u[d];
        uSqr = bgk_collision_base(f, rb, j, L->omega, invRhoOf(rb));
        add_guo_force(f, F, u, L->omega);
        rhoBar = rb;
        break;
    }
    case K_INCBGK:
        get_rhoBar_j(f, &rhoBar, j);
        uSqr = bgk_collision_base(f, rhoBar, j, L->omega, (double)1 / L->rho0);
        break;
    default: /* BGK and the BGK base of every boundary face */
        get_rhoBar_j(f, &rhoBar, j);
        uSqr = bgk_collision_base(f, rhoBar, j, L->omega, invRhoOf(rhoBar));
        break;
    }
    /* latticeStatistics.h:38-43 */
    st->sumRhoBar += rhoBar;
    st->sumUSqr += uSqr;
    if (uSqr > st->maxUSqr) st->maxUSqr = uSqr;
    st->count += 1;
}

/* ExternalRhoJcollideAndStream3D (dynamicsProcessor3D.hh:41-56): every cell's
 * Dynamics::collideExternal with rho-bar and j taken from the fields.  BGK (and
 * the BGK base of boundary cells) and IncBGK run their collision on the given
 * moments and gather no statistics (isoThermalDynamics.hh:333-338, 1422-1427);
 * Guo-forced BGK takes the generic route, shifting every population by the
 * change of equilibrium and then colliding as usual (core/dynamics.hh:131-145);
 * bounce-back, momentum exchange and no-dynamics collide as usual
 * (core/dynamics.hh:793-798, 974-977, bounceBackModels.hh:139-144). */
static void collide_cell_external(const orc_lattice* L, long id, double* f, double rbExt, const double jExt[3],
                                  orc_stats* st) {
    int k = L->flags[id];
    if (k == K_INCBGK) {
        bgk_collision_base(f, rbExt, jExt, L->omega, (double)1 / L->rho0);
        return;
    }
    if (k == K_BGK || (k >= K_REGVEL && k < K_NKINDS)) {
        bgk_collision_base(f, rbExt, jExt, L->omega, invRhoOf(rbExt));
        return;
    }
    if (k == K_GUO) {
        double oldRb, oldJ[3];
        get_rhoBar_j(f, &oldRb, oldJ); /* BasicBulkDynamics::computeRhoBarJ */
        double oldJsqr = oldJ[0] * oldJ[0] + oldJ[1] * oldJ[1] + oldJ[2] * oldJ[2];
        double jSqr = jExt[0] * jExt[0] + jExt[1] * jExt[1] + jExt[2] * jExt[2];
        double oldInv = invRhoOf(oldRb), newInv = invRhoOf(rbExt);
        for (int i = 0; i < 19; ++i) {
            double oldEq = bgk_eq(i, oldRb, oldInv, oldJ, oldJsqr);
            double newEq = bgk_eq(i, rbExt, newInv, jExt, jSqr);
            f[i] += newEq - oldEq;
        }
    }
    collide_cell(L, id, f, st);
}

/* ------------------------------------------------------------ boundary faces */

static int faceDir(int k) { return ((k - K_REGVEL) % 6) / 2; }
static int faceOri(int k) { return (((k - K_REGVEL) % 6) % 2) ? 1 : -1; }
static int faceFamily(int k) { return (k - K_REGVEL) / 6; } /* 0 regvel 1 regpress 2 zhvel 3 zhpress */

/* indexTemplates.h:81-97: indices with c[dir]==value, ascending. */
static int sub_index(int dir, int value, int* out) {
    int n = 0;
    for (int i = 0; i < 19; ++i)
        if (C[i][dir] == value) out[n++] = i;
    return n;
}

/* boundaryDynamics.hh:639-669, VelocityDirichletBoundaryDynamics::computeRhoBar
 * (no external force, velIsJ false for BGK). */
static double vel_face_rhoBar(const double* f, int dir, int ori, const double* vel) {
    int onWall[19], normal[19];
    int nw = sub_index(dir, 0, onWall), nn = sub_index(dir, ori, normal);
    double rhoOnWall = 0., rhoNormal = 0.;
    for (int a = 0; a < nw; ++a) rhoOnWall += f[onWall[a]];
    for (int a = 0; a < nn; ++a) rhoNormal += f[normal[a]];
    double velNormal = (double)ori * (vel[dir] - 0.5 * 0.);
    return ((double)2 * rhoNormal + rhoOnWall - (double)1 * velNormal) / ((double)1 + velNormal);
}

/* boundaryDynamics.hh:683-702 */
static void vel_face_rhoBar_j(const double* f, int dir, int ori, const double* vel, double* rhoBar, double j[3]) {
    *rhoBar = vel_face_rhoBar(f, dir, ori, vel);
    double rho = *rhoBar + (double)1;
    for (int d = 0; d < 3; ++d) j[d] = rho * (vel[d] - 0.5 * 0.);
}

/* boundaryDynamics.hh:775-800 (DensityDirichletBoundaryDynamics::computeJ) and
 * :815-822 (computeRhoBarJ returns the stored rhoBar). */
static void press_face_j(const double* f, int dir, int ori, double rhoBar, double j[3]) {
    int onWall[19], normal[19];
    int nw = sub_index(dir, 0, onWall), nn = sub_index(dir, ori, normal);
    j[0] = j[1] = j[2] = 0.;
    double rhoOnWall = 0., rhoNormal = 0.;
    for (int a = 0; a < nw; ++a) rhoOnWall += f[onWall[a]];
    for (int a = 0; a < nn; ++a) rhoNormal += f[normal[a]];
    j[dir] = (double)ori * ((double)2 * rhoNormal + rhoOnWall - rhoBar);
}

/* offEquilibriumTemplates.h:91-115 (generic form, used by regularize()) */
static double fromPiToFneq(int i, const double Pi[6]) {
    double fNeq = 0.;
    int iPi = 0;
    for (int a = 0; a < 3; ++a) {
        fNeq += Pi[iPi] * ((double)(C[i][a] * C[i][a]) - CS2);
        ++iPi;
        for (int b = a + 1; b < 3; ++b) {
            fNeq += Pi[iPi] * (double)2 * C[i][a] * C[i][b];
            ++iPi;
        }
    }
    fNeq *= T_W[i] * INVCS2 * INVCS2 / (double)2;
    return fNeq;
}

/* regularizedBoundaryDynamics.hh:96-110 / :160-175 with
 * boundaryTemplates.h:42-84 (compute_PiNeq) and isoThermalDynamics.hh:55-69
 * (IsoThermalBulkDynamics::regularize). */
static void regularized_complete(double* f, int dir, int ori, double rhoBar, const double j[3]) {
    double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    double invRho = invRhoOf(rhoBar);
    int onWall[19], normal[19];
    int nw = sub_index(dir, 0, onWall), nn = sub_index(dir, ori, normal);
    double fNeq[19];
    for (int a = 0; a < nw; ++a) {
        int i = onWall[a];
        fNeq[i] = f[i] - bgk_eq(i, rhoBar, invRho, j, jSqr);
    }
    for (int a = 0; a < nn; ++a) {
        int i = normal[a];
        fNeq[i] = (i == 0) ? 0. : f[i] - bgk_eq(i, rhoBar, invRho, j, jSqr);
    }
    double Pi[6];
    int iPi = 0;
    for (int al = 0; al < 3; ++al)
        for (int be = al; be < 3; ++be) {
            double s = 0.;
            for (int a = 0; a < nw; ++a) {
                int i = onWall[a];
                s += (double)(C[i][al] * C[i][be]) * fNeq[i];
            }
            for (int a = 0; a < nn; ++a) {
                int i = normal[a];
                s += (double)2 * C[i][al] * C[i][be] * fNeq[i];
            }
            Pi[iPi++] = s;
        }
    f[0] = bgk_eq(0, rhoBar, invRho, j, jSqr) + fromPiToFneq(0, Pi);
    for (int i = 1; i <= 9; ++i) {
        f[i] = bgk_eq(i, rhoBar, invRho, j, jSqr);
        f[i + 9] = bgk_eq(i + 9, rhoBar, invRho, j, jSqr);
        double fn = fromPiToFneq(i, Pi);
        f[i] += fn;
        f[i + 9] += fn;
    }
}

/* zouHeDynamics.hh:44-113 (ZouHeClosure) */
static void zouhe_complete(double* f, int dir, int ori, double rhoBar, const double j[3]) {
    int normal[19], missing[19], diag[19];
    int nn = sub_index(dir, ori, normal);
    for (int a = 0; a < nn; ++a) missing[a] = opp(normal[a]); /* indexTemplates.h:110-133 */
    int nd = 0, erased = 0;
    for (int a = 0; a < nn; ++a) {
        int p = missing[a];
        int nz = abs(C[p][0]) + abs(C[p][1]) + abs(C[p][2]);
        if (!erased && nz == 1) { erased = 1; continue; }
        diag[nd++] = p;
    }
    double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    double invRho = invRhoOf(rhoBar);
    for (int a = 0; a < nn; ++a) {
        int p = missing[a], o = opp(p);
        f[p] = f[o] - bgk_eq(o, rhoBar, invRho, j, jSqr) + bgk_eq(p, rhoBar, invRho, j, jSqr);
    }
    /* momentTemplates3D.h:410-418 compute_rho_uLb */
    double rb, jj[3], u[3];
    get_rhoBar_j(f, &rb, jj);
    double invR = invRhoOf(rb);
    double falseRho = rb + (double)1;
    for (int d = 0; d < 3; ++d) u[d] = jj[d] * invR;
    double diff[3];
    for (int d = 0; d < 3; ++d) diff[d] = (j[d] - falseRho * u[d]) / (double)nd;
    for (int a = 0; a < nd; ++a) {
        int p = diag[a];
        for (int s = 1; s < 3; ++s) {
            int d = (dir + s) % 3;
            f[p] += (double)C[p][d] * diff[d];
        }
    }
}

/* WrappedLocalBoundaryFunctional3D::process -> prepareCollision ->
 * completePopulations (wrappedLocalBoundaryProcessor3D.hh:43-65). */
static void complete_face(const orc_lattice* L, long id, double* f) {
    int k = L->flags[id];
    int dir = faceDir(k), ori = faceOri(k), fam = faceFamily(k);
    const double* v = L->bcval + 3 * id;
    double rhoBar, j[3];
    if (fam == 0 || fam == 2) {
        vel_face_rhoBar_j(f, dir, ori, v, &rhoBar, j);
    } else {
        rhoBar = v[0] - (double)1; /* StoreDensityDynamics::defineDensity, boundaryDynamics.hh:250-255 */
        press_face_j(f, dir, ori, rhoBar, j);
    }
    if (fam < 2)
        regularized_complete(f, dir, ori, rhoBar, j);
    else
        zouhe_complete(f, dir, ori, rhoBar, j);
}

/* ------------------------------------------------------------ lattice ops */

static inline long lid(const orc_lattice* L, int x, int y, int z) {
    return ((long)x * L->ny + y) * L->nz + z;
}

/* Neighbour of (x,y,z) along c_i (sign s = +1) or -c_i (s = -1).  Returns -1
 * when it leaves a non-periodic domain or lands on a cell outside the lattice.  Periodic axes wrap, which is what the
 * periodic envelope overlaps of MultiBlockLattice3D::collideAndStream
 * (multiBlockLattice3D.hh:318-357, extendPeriodic :253-285) amount to. */
static long neighbour(const orc_lattice* L, int x, int y, int z, int i, int s) {
    int p[3] = {x + s * C[i][0], y + s * C[i][1], z + s * C[i][2]};
    int n[3] = {L->nx, L->ny, L->nz};
    for (int a = 0; a < 3; ++a) {
        if (p[a] < 0 || p[a] >= n[a]) {
            if (!L->periodic[a]) return -1;
            p[a] = (p[a] + n[a]) % n[a];
        }
    }
    long id = lid(L, p[0], p[1], p[2]);
    /* A cell outside every kept block of a sparse domain is treated like the
     * outside of a non-periodic domain. */
    return (L->hasNone && L->flags[id] == K_NONE) ? -1 : id;
}

/* InitializeMomentumExchangeFunctional3D (bounceBackModels3D.hh:42-90): a
 * direction is a fluid direction when the neighbour is neither BounceBack,
 * MomentumExchangeBounceBack nor NoDynamics.  A neighbour outside a
 * non-periodic domain is an envelope cell holding the lattice's background
 * dynamics, which counts as fluid. */
static void build_mebb_masks(orc_lattice* L) {
    for (int x = 0; x < L->nx; ++x)
        for (int y = 0; y < L->ny; ++y)
            for (int z = 0; z < L->nz; ++z) {
                long id = lid(L, x, y, z);
                uint32_t m = 0;
                if (L->flags[id] == K_MEBB) {
                    for (int i = 1; i < 19; ++i) {
                        long nb = neighbour(L, x, y, z, i, +1);
                        int pk = (nb < 0) ? K_BGK : L->flags[nb];
                        if (pk != K_MEBB && pk != K_BB && pk != K_NODYN) m |= 1u << i;
                    }
                }
                L->mebbMask[id] = m;
            }
}

static void complete_edges_corners(const orc_lattice* L, double* f);
static int is_face(int k) { return k >= K_REGVEL && k < K_EDGE; }
static int is_edge(int k) { return k >= K_EDGE && k < K_CORNER; }
static int is_corner(int k) { return k >= K_CORNER && k < K_NKINDS; }

/* One time step: collide every cell, stream (with the swap algorithm's
 * domain-edge rule: a population whose destination lies outside a
 * non-periodic domain stays in the cell, reversed -- blockLattice3D.hh:403-427),
 * then complete the boundary faces. */
static void cell_rhoBar_j(const orc_lattice* L, long id, const double* f, double* rb, double j[3]);

/* extRho / extJ non-null: collide with the external fields (collide_cell_external)
 * and, after streaming, recompute them from the streamed populations before
 * the boundary processors run (BoxRhoBarJfunctional3D integrated at a later
 * processor level, dataAnalysisFunctional3D.hh:528-549) when recompute is set. */
static void step(const orc_lattice* L, double* f, double* tmp, orc_stats* st, double* extRho, double* extJ,
                 int recompute) {
    long n = (long)L->nx * L->ny * L->nz;
    const int external = extRho != NULL;
    double sR = 0., sU = 0., mU = -1.79769313486231570815e+308;
    long cnt = 0;
    double d0 = 0., d1 = 0., d2 = 0.;
#pragma omp parallel for reduction(+ : sR, sU, cnt, d0, d1, d2) reduction(max : mU) schedule(static)
    for (long id = 0; id < n; ++id) {
        orc_stats s = {0., 0., -1.79769313486231570815e+308, 0, {0., 0., 0.}};
        double* c = tmp + id * 19;
        memcpy(c, f + id * 19, 19 * sizeof(double));
        if (external) collide_cell_external(L, id, c, extRho[id], extJ + 3 * id, &s);
        else collide_cell(L, id, c, &s);
        sR += s.sumRhoBar; sU += s.sumUSqr; cnt += s.count;
        if (s.maxUSqr > mU) mU = s.maxUSqr;
        d0 += s.drag[0]; d1 += s.drag[1]; d2 += s.drag[2];
    }
    st->sumRhoBar = sR; st->sumUSqr = sU; st->maxUSqr = mU; st->count = cnt;
    st->drag[0] = d0; st->drag[1] = d1; st->drag[2] = d2;
    const long sx = (long)L->ny * L->nz, sy = L->nz;
    long dlt[19];
    for (int i = 0; i < 19; ++i) dlt[i] = C[i][0] * sx + C[i][1] * sy + C[i][2];
#pragma omp parallel for collapse(2) schedule(static)
    for (int x = 0; x < L->nx; ++x)
        for (int y = 0; y < L->ny; ++y) {
            const int inner = !L->hasNone && x > 0 && x < L->nx - 1 && y > 0 && y < L->ny - 1;
            for (int z = 0; z < L->nz; ++z) {
                long id = lid(L, x, y, z);
                double* out = f + id * 19;
                if (L->hasNone && L->flags[id] == K_NONE) {
                    for (int i = 0; i < 19; ++i) out[i] = 0.;
                    continue;
                }
                out[0] = tmp[id * 19];
                if (inner && z > 0 && z < L->nz - 1) {
                    /* no source lies outside the box: plain offsets */
                    for (int i = 1; i < 19; ++i) out[i] = tmp[(id - dlt[i]) * 19 + i];
                } else {
                    for (int i = 1; i < 19; ++i) {
                        long src = neighbour(L, x, y, z, i, -1);
                        out[i] = (src >= 0) ? tmp[src * 19 + i] : tmp[id * 19 + opp(i)];
                    }
                }
                if (!external && is_face(L->flags[id])) complete_face(L, id, out);
            }
        }
    if (external) {
        if (recompute)
#pragma omp parallel for schedule(static)
            for (long id = 0; id < n; ++id) cell_rhoBar_j(L, id, f + id * 19, extRho + id, extJ + 3 * id);
        for (long id = 0; id < n; ++id)
            if (is_face(L->flags[id])) complete_face(L, id, f + id * 19);
    }
    if (L->hasEdges) complete_edges_corners(L, f);
}

/* ------------------------------------------------------------ public API */

typedef struct {
    int nx, ny, nz;
    int periodic[3];
    double omega, rho0, bbRho;
} orc_params;

static void setup(orc_lattice* L, const orc_params* p, const uint8_t* flags, const double* bcval,
                  const double* force) {
    init_constants();
    L->nx = p->nx; L->ny = p->ny; L->nz = p->nz;
    for (int a = 0; a < 3; ++a) L->periodic[a] = p->periodic[a];
    L->omega = p->omega; L->rho0 = p->rho0; L->bbRho = p->bbRho;
    L->flags = flags; L->bcval = bcval; L->force = force;
    long n = (long)p->nx * p->ny * p->nz;
    L->hasNone = 0;
    for (long id = 0; id < n; ++id)
        if (flags[id] == K_NONE) { L->hasNone = 1; break; }
    L->mebbMask = (uint32_t*)calloc((size_t)n, sizeof(uint32_t));
    build_mebb_masks(L);
    L->hasEdges = 0;
    for (long id = 0; id < n; ++id)
        if (flags[id] >= K_EDGE && flags[id] < K_NKINDS) { L->hasEdges = 1; break; }
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Complete the boundary faces in place: MultiBlock3D::initialize() runs the
 * boundary processors once (multiBlock3D.cpp:330-332). */
int orc_initialize(const orc_params* p, const uint8_t* flags, const double* bcval,
                   const double* force, double* f) {
    orc_lattice L;
    setup(&L, p, flags, bcval, force);
    long n = (long)p->nx * p->ny * p->nz;
    for (long id = 0; id < n; ++id)
        if (is_face(flags[id])) complete_face(&L, id, f + id * 19);
    if (L.hasEdges) complete_edges_corners(&L, f);
    free(L.mebbMask);
    return 0;
}

/* Run nsteps collideAndStream() steps in place on f ([x][y][z][19]).
 * stats (optional, nsteps*7 doubles): per step avRhoBar, avUSqr, maxUSqr,
 * drag x/y/z, stat-cell count -- the values BlockStatistics::evaluate()
 * publishes after each step (core/blockStatistics.cpp:77-110). */
int orc_run(const orc_params* p, const uint8_t* flags, const double* bcval, const double* force,
            double* f, int nsteps, double* stats) {
    orc_lattice L;
    setup(&L, p, flags, bcval, force);
    long n = (long)p->nx * p->ny * p->nz;
    double* tmp = (double*)malloc((size_t)n * 19 * sizeof(double));
    if (!tmp) { free(L.mebbMask); return -1; }
    for (int s = 0; s < nsteps; ++s) {
        orc_stats st;
        step(&L, f, tmp, &st, NULL, NULL, 0);
        if (stats) {
            double* r = stats + 7 * (long)s;
            r[0] = st.count ? st.sumRhoBar / (double)st.count : 0.;
            r[1] = st.count ? st.sumUSqr / (double)st.count : 0.;
            r[2] = st.maxUSqr;
            r[3] = st.drag[0]; r[4] = st.drag[1]; r[5] = st.drag[2];
            r[6] = (double)st.count;
        }
    }
    free(tmp);
    free(L.mebbMask);
    return 0;
}

/* Per-cell velocity the way Cell::computeVelocity dispatches it. */
static void cell_velocity(const orc_lattice* L, long id, const double* f, double u[3]) {
    int k = L->flags[id];
    double rb, j[3];
    switch (k) {
    case K_BB: case K_MEBB: case K_NODYN: case K_NONE:
        u[0] = u[1] = u[2] = 0.; /* core/dynamics.hh:824-829, bounceBackModels.hh:170-175 */
        return;
    case K_GUO: { /* externalForceDynamics.hh:58-73 */
        const double* F = L->force + 3 * id;
        get_rhoBar_j(f, &rb, j);
        double invRho = invRhoOf(rb);
        for (int d = 0; d < 3; ++d) u[d] = j[d] * invRho + F[d] / (double)2;
        return;
    }
    case K_INCBGK: /* isoThermalDynamics.hh:1388-1395 */
        get_rhoBar_j(f, &rb, j);
        for (int d = 0; d < 3; ++d) u[d] = j[d] * ((double)1 / L->rho0);
        return;
    case K_BGK: { /* momentTemplates3D.h:402-408 compute_uLb */
        get_j(f, j);
        double invRho = invRhoOf(get_rhoBar(f));
        for (int d = 0; d < 3; ++d) u[d] = j[d] * invRho;
        return;
    }
    default: break;
    }
    const double* v = L->bcval + 3 * id;
    if (k >= K_EDGE) { /* StoreVelocityDynamics::computeVelocity */
        for (int d = 0; d < 3; ++d) u[d] = v[d];
        return;
    }
    int fam = faceFamily(k), dir = faceDir(k), ori = faceOri(k);
    if (fam == 0 || fam == 2) { /* StoreVelocityDynamics::computeVelocity, boundaryDynamics.hh:324-330 */
        for (int d = 0; d < 3; ++d) u[d] = v[d];
        return;
    }
    /* DensityDirichletBoundaryDynamics::computeVelocity, boundaryDynamics.hh:790-812 */
    double rhoBar = v[0] - (double)1;
    press_face_j(f, dir, ori, rhoBar, u);
    double invRho = invRhoOf(rhoBar);
    for (int d = 0; d < 3; ++d) { u[d] *= invRho; u[d] += 0.5 * 0.; }
}

static double cell_rhoBar(const orc_lattice* L, long id, const double* f) {
    int k = L->flags[id];
    switch (k) {
    case K_BB: case K_MEBB: return L->bbRho - (double)1; /* core/dynamics.hh:875-877 */
    case K_NODYN: return (double)1 - (double)1;          /* core/dynamics.hh:1055-1058 */
    case K_BGK: case K_GUO: case K_INCBGK: return get_rhoBar(f); /* core/dynamics.hh:351-354 */
    default: break;
    }
    /* StoreVelocityDynamics::computeRhoBar: rhoBar(computeDensity()) with the BGK
     * base density (boundaryDynamics.hh:342-345) */
    if (k >= K_EDGE) return (get_rhoBar(f) + (double)1) - (double)1;
    int fam = faceFamily(k);
    if (fam == 0 || fam == 2) return vel_face_rhoBar(f, faceDir(k), faceOri(k), L->bcval + 3 * id);
    return L->bcval[3 * id] - (double)1; /* StoreDensityDynamics::computeRhoBar */
}

/* ------------------------------------------------------------ edges and corners
 *
 * External velocity edges and corners of createLocalBoundaryCondition3D:
 * StoreVelocityDynamics around the BGK base, completed by the finite-
 * difference processors OuterVelocityEdgeFunctional3D /
 * OuterVelocityCornerFunctional3D (finiteDifferenceBoundaryProcessor3D.hh:
 * 141-316), which run after the face processors and before each other in the
 * order faces, edges, corners (setVelocityConditionOnBlockBoundaries,
 * boundaryCondition3D.hh:65-163). */

/* Density the way Cell::computeDensity reports it. */
static double cell_density(const orc_lattice* L, long id, const double* f) {
    int k = L->flags[id];
    switch (k) {
    /* BounceBack / NoDynamics return their rho member (core/dynamics.hh:814-816,
     * 994-996), constructed here with bbRho */
    case K_BB: case K_MEBB: case K_NODYN: return L->bbRho;
    case K_BGK: case K_GUO: case K_INCBGK: return get_rhoBar(f) + (double)1; /* compute_rho */
    default: break;
    }
    if (k >= K_EDGE) return get_rhoBar(f) + (double)1; /* BoundaryCompositeDynamics -> base */
    int fam = faceFamily(k);
    if (fam == 0 || fam == 2) return vel_face_rhoBar(f, faceDir(k), faceOri(k), L->bcval + 3 * id) + (double)1;
    return (L->bcval[3 * id] - (double)1) + (double)1; /* StoreDensityDynamics::computeDensity */
}

/* f-bar of the IsoThermalBulkDynamics::regularize (isoThermalDynamics.hh:55-69)
 * with the BGK equilibrium and offEquilibriumTemplates::fromPiToFneq. */
static void regularize_pi(double* f, double rhoBar, const double j[3], double jSqr, const double Pi[6]) {
    double invRho = invRhoOf(rhoBar);
    f[0] = bgk_eq(0, rhoBar, invRho, j, jSqr) + fromPiToFneq(0, Pi);
    for (int i = 1; i <= 9; ++i) {
        f[i] = bgk_eq(i, rhoBar, invRho, j, jSqr);
        f[i + 9] = bgk_eq(i + 9, rhoBar, invRho, j, jSqr);
        double fn = fromPiToFneq(i, Pi);
        f[i] += fn;
        f[i + 9] += fn;
    }
}

static void velocity_at(const orc_lattice* L, const double* f, int x, int y, int z, double u[3]) {
    long id = lid(L, x, y, z);
    cell_velocity(L, id, f + id * 19, u);
}

static double density_at(const orc_lattice* L, const double* f, int x, int y, int z) {
    long id = lid(L, x, y, z);
    return cell_density(L, id, f + id * 19);
}

/* fd::DirectedGradients3D (finiteDifference/finiteDifference3D.h:61-190):
 * o1 forward difference along the boundary normal, central difference along
 * the boundary. */
static void grad_normal(const orc_lattice* L, const double* f, int p[3], int dir, int ori, double g[3]) {
    double u0[3], u1[3];
    velocity_at(L, f, p[0], p[1], p[2], u0);
    int q[3] = {p[0], p[1], p[2]};
    q[dir] -= ori;
    velocity_at(L, f, q[0], q[1], q[2], u1);
    for (int d = 0; d < 3; ++d) g[d] = (double)(-ori) * (-u0[d] + u1[d]); /* fdStencils1D.h:58-60 */
}

static void grad_central(const orc_lattice* L, const double* f, int p[3], int dir, double g[3]) {
    double up[3], um[3];
    int a[3] = {p[0], p[1], p[2]}, b[3] = {p[0], p[1], p[2]};
    a[dir] += 1;
    b[dir] -= 1;
    velocity_at(L, f, a[0], a[1], a[2], up);
    velocity_at(L, f, b[0], b[1], b[2], um);
    for (int d = 0; d < 3; ++d) g[d] = (up[d] - um[d]) / (double)2; /* fdStencils1D.h:39-42 */
}

/* pi from the velocity gradients dA_uB[A][B] = d_A u_B and rho
 * (finiteDifferenceBoundaryProcessor3D.hh:180-191). */
static void pi_from_gradients(double dAuB[3][3], double rho, double omega, double Pi[6]) {
    double sToPi = -rho / INVCS2 / omega;
    Pi[0] = (double)2 * dAuB[0][0] * sToPi;
    Pi[3] = (double)2 * dAuB[1][1] * sToPi;
    Pi[5] = (double)2 * dAuB[2][2] * sToPi;
    Pi[1] = (dAuB[0][1] + dAuB[1][0]) * sToPi;
    Pi[2] = (dAuB[0][2] + dAuB[2][0]) * sToPi;
    Pi[4] = (dAuB[1][2] + dAuB[2][1]) * sToPi;
}

static void complete_edge(const orc_lattice* L, double* f, int x, int y, int z) {
    long id = lid(L, x, y, z);
    int e = L->flags[id] - K_EDGE;
    int plane = e / 4, n1 = (e & 2) ? 1 : -1, n2 = (e & 1) ? 1 : -1;
    int d1 = (plane + 1) % 3, d2 = (plane + 2) % 3;
    int p[3] = {x, y, z};
    /* getNeighborRho (finiteDifferenceBoundaryProcessor3D.hh:220-227) */
    int a[3] = {x, y, z}, b[3] = {x, y, z};
    a[d1] -= n1;
    b[d2] -= n2;
    double rho10 = density_at(L, f, a[0], a[1], a[2]);
    double rho01 = density_at(L, f, b[0], b[1], b[2]);
    double rho = (double)0.5 * (rho01 + rho10);
    double dAuB[3][3];
    grad_central(L, f, p, plane, dAuB[plane]);
    grad_normal(L, f, p, d1, n1, dAuB[d1]);
    grad_normal(L, f, p, d2, n2, dAuB[d2]);
    double Pi[6];
    pi_from_gradients(dAuB, rho, L->omega, Pi);
    double vel[3], j[3];
    cell_velocity(L, id, f + id * 19, vel);
    for (int d = 0; d < 3; ++d) j[d] = rho * vel[d];
    double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    regularize_pi(f + id * 19, rho - (double)1, j, jSqr, Pi);
}

static void complete_corner(const orc_lattice* L, double* f, int x, int y, int z) {
    long id = lid(L, x, y, z);
    int c = L->flags[id] - K_CORNER;
    int nx = (c & 4) ? 1 : -1, ny = (c & 2) ? 1 : -1, nz = (c & 1) ? 1 : -1;
    double rho100 = density_at(L, f, x - nx, y, z);
    double rho010 = density_at(L, f, x, y - ny, z);
    double rho001 = density_at(L, f, x, y, z - nz);
    double rho = (double)1 / (double)3 * (rho001 + rho010 + rho100);
    int p[3] = {x, y, z};
    double dAuB[3][3];
    grad_normal(L, f, p, 0, nx, dAuB[0]);
    grad_normal(L, f, p, 1, ny, dAuB[1]);
    grad_normal(L, f, p, 2, nz, dAuB[2]);
    double Pi[6];
    pi_from_gradients(dAuB, rho, L->omega, Pi);
    double vel[3], j[3];
    cell_velocity(L, id, f + id * 19, vel);
    for (int d = 0; d < 3; ++d) j[d] = rho * vel[d];
    double jSqr = j[0] * j[0] + j[1] * j[1] + j[2] * j[2];
    regularize_pi(f + id * 19, rho - (double)1, j, jSqr, Pi);
}

/* The non-local post-stream processors: edges, then corners. */
static void complete_edges_corners(const orc_lattice* L, double* f) {
    for (int pass = 0; pass < 2; ++pass)
        for (int x = 0; x < L->nx; ++x)
            for (int y = 0; y < L->ny; ++y)
                for (int z = 0; z < L->nz; ++z) {
                    int k = L->flags[lid(L, x, y, z)];
                    if (pass == 0 && is_edge(k)) complete_edge(L, f, x, y, z);
                    if (pass == 1 && is_corner(k)) complete_corner(L, f, x, y, z);
                }
}

/* Dynamics::computeRhoBarJ the way each kind implements it: the bulk moments
 * (core/dynamics.hh:357-361), the stored rho of bounce-back / momentum
 * exchange with j = 0 (core/dynamics.hh:880-885, bounceBackModels.hh:226-231),
 * rho-bar 0 and j = 0 for no-dynamics (core/dynamics.hh:1061-1066), the
 * velocity-face and pressure-face formulas (boundaryDynamics.hh:682-702,
 * 815-822) and, for edges and corners, the base density with the stored
 * velocity (boundaryDynamics.hh:348-360). */
static void cell_rhoBar_j(const orc_lattice* L, long id, const double* f, double* rb, double j[3]) {
    int k = L->flags[id];
    const double* v = L->bcval + 3 * id;
    switch (k) {
    case K_BB: case K_MEBB:
        *rb = L->bbRho - (double)1;
        j[0] = j[1] = j[2] = 0.;
        return;
    case K_NODYN:
        *rb = (double)1 - (double)1;
        j[0] = j[1] = j[2] = 0.;
        return;
    case K_BGK: case K_GUO: case K_INCBGK:
        get_rhoBar_j(f, rb, j);
        return;
    default: break;
    }
    if (k >= K_EDGE) {
        double rho = get_rhoBar(f) + (double)1;
        *rb = rho - (double)1;
        for (int d = 0; d < 3; ++d) j[d] = rho * (v[d] - 0.5 * 0.);
        return;
    }
    int fam = faceFamily(k), dir = faceDir(k), ori = faceOri(k);
    if (fam == 0 || fam == 2) {
        vel_face_rhoBar_j(f, dir, ori, v, rb, j);
    } else {
        *rb = v[0] - (double)1;
        press_face_j(f, dir, ori, *rb, j);
    }
}

/* BoxRhoBarJfunctional3D over the bounding box: rho-bar (N) and j (N*3). */
int orc_rhobar_j(const orc_params* p, const uint8_t* flags, const double* bcval, const double* force,
                 const double* f, double* rhoBar, double* j) {
    orc_lattice L;
    setup(&L, p, flags, bcval, force);
    long n = (long)p->nx * p->ny * p->nz;
    for (long id = 0; id < n; ++id) cell_rhoBar_j(&L, id, f + id * 19, rhoBar + id, j + 3 * id);
    free(L.mebbMask);
    return 0;
}

/* nsteps of ExternalRhoJcollideAndStream3D with the fields rhoBar / j (updated
 * in place when recompute is set); stats as orc_run (drag only: the BGK-family
 * external collisions gather none). */
int orc_run_external(const orc_params* p, const uint8_t* flags, const double* bcval, const double* force,
                     double* f, double* rhoBar, double* j, int recompute, int nsteps, double* stats) {
    orc_lattice L;
    setup(&L, p, flags, bcval, force);
    long n = (long)p->nx * p->ny * p->nz;
    double* tmp = (double*)malloc((size_t)n * 19 * sizeof(double));
    if (!tmp) { free(L.mebbMask); return -1; }
    for (int s = 0; s < nsteps; ++s) {
        orc_stats st;
        step(&L, f, tmp, &st, rhoBar, j, recompute);
        if (stats) {
            double* r = stats + 7 * (long)s;
            r[0] = st.count ? st.sumRhoBar / (double)st.count : 0.;
            r[1] = st.count ? st.sumUSqr / (double)st.count : 0.;
            r[2] = st.maxUSqr; /* the lowest double when no cell gathered statistics */
            r[3] = st.drag[0]; r[4] = st.drag[1]; r[5] = st.drag[2];
            r[6] = (double)st.count;
        }
    }
    free(tmp);
    free(L.mebbMask);
    return 0;
}

/* computeAverageEnergy / computeAverageDensity over the bounding box
 * (dataAnalysisWrapper3D.hh:1226-1262, dataAnalysisFunctional3D.hh:57-123). */
int orc_reduce(const orc_params* p, const uint8_t* flags, const double* bcval, const double* force,
               const double* f, double* energy, double* density) {
    orc_lattice L;
    setup(&L, p, flags, bcval, force);
    long n = (long)p->nx * p->ny * p->nz;
    double sE = 0., sR = 0.;
    long cells = 0;   /* cells of the lattice (a sparse domain averages over its kept blocks) */
    for (long id = 0; id < n; ++id) {
        if (flags[id] == K_NONE) continue;
        double u[3];
        cell_velocity(&L, id, f + id * 19, u);
        sE += u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        sR += cell_rhoBar(&L, id, f + id * 19);
        ++cells;
    }
    *energy = sE / (double)2 / (double)cells;
    *density = sR / (double)cells + (double)1;
    free(L.mebbMask);
    return 0;
}

/* computeVelocity of every cell (3 doubles per cell). */
int orc_velocity(const orc_params* p, const uint8_t* flags, const double* bcval, const double* force,
                 const double* f, double* u) {
    orc_lattice L;
    setup(&L, p, flags, bcval, force);
    long n = (long)p->nx * p->ny * p->nz;
    for (long id = 0; id < n; ++id) cell_velocity(&L, id, f + id * 19, u + 3 * id);
    free(L.mebbMask);
    return 0;
}

/* Expose the fluid-direction masks (for tests of the device-side masks). */
int orc_mebb_masks(const orc_params* p, const uint8_t* flags, uint32_t* out) {
    orc_lattice L;
    setup(&L, p, flags, NULL, NULL);
    long n = (long)p->nx * p->ny * p->nz;
    memcpy(out, L.mebbMask, (size_t)n * sizeof(uint32_t));
    free(L.mebbMask);
    return 0;
}

/* computeSparseManagement (offLattice/makeSparse3D.hh:47-160) over the
 * regular block distribution createRegularDistribution3D(nx, ny, nz, bx, by,
 * bz) (multiBlock/staticRepartitions3D.cpp:38-63, the first n % b blocks of an
 * axis one cell longer): a block is kept when any cell of its bulk has a
 * non-zero field value.  keep[(ix * by + iy) * bz + iz]; returns the number of
 * kept blocks. */
static void regular_ranges(int n, int b, int* start) {
    int pos = 0;
    for (int i = 0; i < b; ++i) {
        start[i] = pos;
        pos += n / b + (i < n % b ? 1 : 0);
    }
    start[b] = pos;
}

int orc_sparse_blocks(int nx, int ny, int nz, const int32_t* field, int bx, int by, int bz, uint8_t* keep) {
    int sx[bx + 1], sy[by + 1], sz[bz + 1];
    regular_ranges(nx, bx, sx);
    regular_ranges(ny, by, sy);
    regular_ranges(nz, bz, sz);
    int kept = 0;
    for (int ix = 0; ix < bx; ++ix)
        for (int iy = 0; iy < by; ++iy)
            for (int iz = 0; iz < bz; ++iz) {
                int any = 0;
                for (int x = sx[ix]; x < sx[ix + 1] && !any; ++x)
                    for (int y = sy[iy]; y < sy[iy + 1] && !any; ++y)
                        for (int z = sz[iz]; z < sz[iz + 1]; ++z)
                            if (field[((long)x * ny + y) * nz + z] != 0) { any = 1; break; }
                keep[(ix * by + iy) * bz + iz] = (uint8_t)any;
                kept += any;
            }
    return kept;
}


/* ------------------------------------------------------------ mesh voxelizer
 *
 * voxelize(mesh, domain, borderWidth) (offLattice/voxelizer.hh:106-141): the
 * outer layer of the box is seeded "outside", every other cell starts
 * undetermined; sweeps of VoxelizeMeshFunctional3D give an undetermined cell
 * the flag of a determined neighbour (any of the 26), inverted when the
 * segment between their centres crosses the surface an odd number of times
 * (voxelizer.hh:330-380, checkIfFacetsCrossed :259-310), until no cell is
 * undetermined; DetectBorderLineFunctional3D (:653-685) then marks outside
 * cells with an inside cell within borderWidth as outerBorder and inside
 * cells with an outside one as innerBorder.
 *
 * The segment test restates TriangularSurfaceMesh::pointOnTriangle with
 * flag 0 (triangularSurfaceMesh.hh:1022-1120): tolerance eps1 = 100 DBL_EPSILON;
 * an end point on the triangle's plane shifts the triangle by 2 eps1 along
 * its unit normal (so a cell centre on the surface lies behind it); a
 * segment parallel to the plane does not cross.  The crossings of a segment
 * are counted as distinct distances (equal within 1e4 DBL_EPSILON, the
 * reference's merge tolerance), after sorting them; the reference compares
 * them in the order its triangle hash lists them.
 *
 * Flags: 1 outside, 2 outerBorder, 3 inside, 4 innerBorder.  The check of a
 * whole mesh against every segment is brute force (with a bounding-box
 * rejection): test infrastructure for boxes of some 10^5 cells. */

enum { VX_UNDET = 0, VX_OUT = 1, VX_OUTB = 2, VX_IN = 3, VX_INB = 4 };

static int vx_inside(int f) { return f == VX_IN || f == VX_INB; }
static int vx_outside(int f) { return f == VX_OUT || f == VX_OUTB; }

static double vx_dot(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* pointOnTriangle(p1, p2, flag 0): 1 and the distance from p1 when the
 * segment p1-p2 meets the triangle (boundary included), else 0. */
static int vx_segment_hits(const double* tri, const double* p1, const double* p2, double* dist) {
    const double eps1 = 100.0 * 2.220446049250313e-16;
    double v0[3] = {tri[0], tri[1], tri[2]};
    double e0[3], e1[3], n[3], dir[3];
    for (int d = 0; d < 3; ++d) {
        e0[d] = tri[3 + d] - tri[d];
        e1[d] = tri[6 + d] - tri[d];
        dir[d] = p2[d] - p1[d];
    }
    n[0] = e0[1] * e1[2] - e0[2] * e1[1];
    n[1] = e0[2] * e1[0] - e0[0] * e1[2];
    n[2] = e0[0] * e1[1] - e0[1] * e1[0];
    const double nn = sqrt(vx_dot(n, n));
    for (int d = 0; d < 3; ++d) n[d] /= nn;
    double num = vx_dot(v0, n) - vx_dot(p1, n);
    const double denom = vx_dot(dir, n);
    double t = num / denom;
    if (fabs(t) <= eps1 || fabs(t - 1.0) <= eps1) {
        for (int d = 0; d < 3; ++d) v0[d] += 2.0 * eps1 * n[d];
        num = vx_dot(v0, n) - vx_dot(p1, n);
        t = num / denom;
    }
    if (fabs(denom) <= eps1) return 0;   /* parallel (or in the plane): no crossing counted */
    if ((t < 0.0 && fabs(t) > eps1) || (t > 1.0 && fabs(t - 1.0) > eps1)) return 0;
    double x[3], tmp[3];
    for (int d = 0; d < 3; ++d) {
        x[d] = p1[d] + dir[d] * t;
        tmp[d] = x[d] - v0[d];
    }
    const double a00 = vx_dot(e0, e0), a01 = vx_dot(e0, e1), a11 = vx_dot(e1, e1);
    const double b0 = vx_dot(tmp, e0), b1 = vx_dot(tmp, e1);
    const double det = a00 * a11 - a01 * a01;
    const double u = (a11 * b0 - a01 * b1) / det;
    const double v = (a00 * b1 - a01 * b0) / det;
    const double upv = u + v;
    if ((u < 0.0 && fabs(u) > eps1) || (u > 1.0 && fabs(u - 1.0) > eps1) || (v < 0.0 && fabs(v) > eps1) ||
        (v > 1.0 && fabs(v - 1.0) > eps1) || (upv > 1.0 && fabs(upv - 1.0) > eps1))
        return 0;
    *dist = fabs(t) * sqrt(vx_dot(dir, dir));
    return 1;
}

static int vx_cmp(const void* a, const void* b) {
    const double x = *(const double*)a, y = *(const double*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* checkIfFacetsCrossed: an odd number of distinct crossings. */
static int vx_crossed(const double* tri, long ntri, const double* lo, const double* hi, const double* p1,
                      const double* p2, double* buf) {
    int m = 0;
    for (long k = 0; k < ntri; ++k) {
        const double* T = tri + 9 * k;
        int skip = 0;
        for (int d = 0; d < 3 && !skip; ++d) {
            const double smin = p1[d] < p2[d] ? p1[d] : p2[d], smax = p1[d] < p2[d] ? p2[d] : p1[d];
            if (hi[3 * k + d] < smin - 1e-9 || lo[3 * k + d] > smax + 1e-9) skip = 1;
        }
        double dist;
        if (!skip && vx_segment_hits(T, p1, p2, &dist) && m < 256) buf[m++] = dist;
    }
    if (m == 0) return 0;
    qsort(buf, (size_t)m, sizeof(double), vx_cmp);
    int distinct = 1;
    for (int i = 1; i < m; ++i)
        if (fabs(buf[i] - buf[i - 1]) > 1e4 * 2.220446049250313e-16) ++distinct;
    return distinct & 1;
}

int orc_voxelize(const double* tri, long ntri, int nx, int ny, int nz, int borderWidth, int32_t* flags) {
    const long n = (long)nx * ny * nz;
    double* lo = (double*)malloc(sizeof(double) * 3 * (size_t)(ntri > 0 ? ntri : 1));
    double* hi = (double*)malloc(sizeof(double) * 3 * (size_t)(ntri > 0 ? ntri : 1));
    int32_t* bulk = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    double buf[256];
    if (!lo || !hi || !bulk) {
        free(lo); free(hi); free(bulk);
        return -1;
    }
    for (long k = 0; k < ntri; ++k)
        for (int d = 0; d < 3; ++d) {
            double a = tri[9 * k + d], b = tri[9 * k + 3 + d], c = tri[9 * k + 6 + d];
            lo[3 * k + d] = fmin(a, fmin(b, c));
            hi[3 * k + d] = fmax(a, fmax(b, c));
        }
    for (int x = 0; x < nx; ++x)
        for (int y = 0; y < ny; ++y)
            for (int z = 0; z < nz; ++z) {
                const int edge = x == 0 || y == 0 || z == 0 || x == nx - 1 || y == ny - 1 || z == nz - 1;
                bulk[((long)x * ny + y) * nz + z] = edge ? VX_OUT : VX_UNDET;
            }
    int changed = 1;
    while (changed) {
        changed = 0;
        for (int x = 1; x < nx - 1; ++x)
            for (int y = 1; y < ny - 1; ++y)
                for (int z = 1; z < nz - 1; ++z) {
                    const long id = ((long)x * ny + y) * nz + z;
                    if (bulk[id] != VX_UNDET) continue;
                    for (int k = 0; k < 27 && bulk[id] == VX_UNDET; ++k) {
                        const int dx = k / 9 - 1, dy = (k / 3) % 3 - 1, dz = k % 3 - 1;
                        if (!dx && !dy && !dz) continue;
                        const int nb = bulk[((long)(x + dx) * ny + (y + dy)) * nz + (z + dz)];
                        if (nb == VX_UNDET) continue;
                        const double p1[3] = {x, y, z}, p2[3] = {x + dx, y + dy, z + dz};
                        const int c = vx_crossed(tri, ntri, lo, hi, p1, p2, buf);
                        bulk[id] = c ? (nb == VX_IN ? VX_OUT : VX_IN) : nb;
                        changed = 1;
                    }
                }
    }
    for (int x = 0; x < nx; ++x)
        for (int y = 0; y < ny; ++y)
            for (int z = 0; z < nz; ++z) {
                const long id = ((long)x * ny + y) * nz + z;
                int f = bulk[id];
                for (int dx = -borderWidth; dx <= borderWidth; ++dx)
                    for (int dy = -borderWidth; dy <= borderWidth; ++dy)
                        for (int dz = -borderWidth; dz <= borderWidth; ++dz) {
                            if (!dx && !dy && !dz) continue;
                            const int X = x + dx, Y = y + dy, Z = z + dz;
                            if (X < 0 || Y < 0 || Z < 0 || X >= nx || Y >= ny || Z >= nz) continue;
                            const int g = bulk[((long)X * ny + Y) * nz + Z];
                            if (vx_outside(bulk[id]) && vx_inside(g)) f = VX_OUTB;
                            if (vx_inside(bulk[id]) && vx_outside(g)) f = VX_INB;
                        }
                flags[id] = f;
            }
    free(lo);
    free(hi);
    free(bulk);
    return 0;
}
