/*
 * plbgpu -- C ABI of the GB300 D3Q19 lattice library.
 *
 * One context drives one GPU through one CUDA stream.  A context owns any
 * number of domains; a domain is one rectangular D3Q19 lattice (the bounding
 * box of a MultiBlockLattice3D, or one block handed to a co-processor) held in
 * a single device allocation.  Every call is synchronous with respect to the
 * host unless stated otherwise, takes plain pointers and sizes, and returns an
 * int status: PLBGPU_OK (0) or a negative PLBGPU_ERR_* code; the message of
 * the last failure is available from plbgpu_last_error().  No C++ exception
 * crosses this interface.
 *
 * Populations cross the interface as f-bar = f - t_i (the reference's stored
 * representation, latticeBoltzmann/roundOffPolicy.h:40-89) in FP64, in the
 * co-processor transfer layout: z fastest, then y, then x, and the 19
 * populations of a cell contiguous in the D3Q19 order of
 * latticeBoltzmann/nearestNeighborLattices3D.hh:168-180
 * (coProcessors/coProcessor3D.h:84-91).
 *
 * Reference paths in the comments are relative to the reference's src/.
 */
#ifndef PLBGPU_H
#define PLBGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct plbgpu_ctx plbgpu_ctx;

/* Status codes. */
#define PLBGPU_OK 0
#define PLBGPU_ERR_ARG (-1)      /* bad argument (size, box, kind, precision) */
#define PLBGPU_ERR_HANDLE (-2)   /* unknown domain handle */
#define PLBGPU_ERR_CUDA (-3)     /* CUDA runtime error */
#define PLBGPU_ERR_NOMEM (-4)    /* device allocation failed */
#define PLBGPU_ERR_STATE (-5)    /* call not valid in the domain's current state */

/* Storage precision of the populations.  FP64 computes in FP64 and
 * reproduces the reference bit for bit; the other forms compute in FP32 and
 * store f-bar in FP32, BF16 or FP16 (the FP64 reductions are kept). */
#define PLBGPU_FP64 0
#define PLBGPU_FP32 1
#define PLBGPU_BF16 2
#define PLBGPU_FP16 3
/* BF16 storage written with stochastic rounding (zero-mean rounding error;
 * reproducible: the random bits hash the slot address and the step count). */
#define PLBGPU_BF16_SR 4

/* Cell kinds (dynamics) -- one byte per cell.  Face kinds are
 * base + 2*direction + (orientation > 0 ? 1 : 0). */
#define PLBGPU_BGK 0          /* BGKdynamics, basicDynamics/isoThermalDynamics.hh:319-330 */
#define PLBGPU_GUO 1          /* GuoExternalForceBGKdynamics, basicDynamics/externalForceDynamics.hh:215-234 */
#define PLBGPU_INCBGK 2       /* IncBGKdynamics, basicDynamics/isoThermalDynamics.hh:1408-1419 */
#define PLBGPU_BOUNCEBACK 3   /* BounceBack, core/dynamics.hh:783-790 */
#define PLBGPU_MOMENTUM_EXCHANGE 4 /* MomentumExchangeBounceBack, boundaryCondition/bounceBackModels.hh:100-136 */
#define PLBGPU_NODYNAMICS 5   /* NoDynamics, core/dynamics.hh:968-971 */
#define PLBGPU_REG_VELOCITY 6 /* RegularizedVelocityBoundaryDynamics (wrapped), regularizedBoundaryDynamics.hh:96-110 */
#define PLBGPU_REG_PRESSURE 12 /* RegularizedDensityBoundaryDynamics (wrapped), regularizedBoundaryDynamics.hh:160-175 */
#define PLBGPU_ZOUHE_VELOCITY 18 /* ZouHeVelocityDynamics (wrapped), zouHeDynamics.hh:44-113, 166-169 */
#define PLBGPU_ZOUHE_PRESSURE 24 /* ZouHePressureDynamics (wrapped), zouHeDynamics.hh:222-225 */
/* External velocity edge of the local regularized condition along axis
 * `plane`, base + 4*plane + 2*(normal1 > 0) + (normal2 > 0) with normal1 along
 * (plane+1)%3 and normal2 along (plane+2)%3: StoreVelocityDynamics around BGK,
 * finished after every step (and by plbgpu_initialize) by the finite-difference
 * OuterVelocityEdgeFunctional3D (boundaryInstantiator3D.h:423-470,
 * finiteDifferenceBoundaryProcessor3D.hh:145-228). */
#define PLBGPU_VELOCITY_EDGE 30
/* External velocity corner, base + 4*(xNormal > 0) + 2*(yNormal > 0) +
 * (zNormal > 0): OuterVelocityCornerFunctional3D, run after the edges
 * (finiteDifferenceBoundaryProcessor3D.hh:238-316). */
#define PLBGPU_VELOCITY_CORNER 42

/* ------------------------------------------------------------ context */

/* Create a context on CUDA device `device`.  Replaces the singleton
 * global::defaultCoProcessor3D<T>() (coProcessors/coProcessor3D.h:178-186).
 * Environment variables read here: PLBGPU_STAGED_TRANSFERS=1 (see
 * plbgpu_send) and PLBGPU_ROW_KERNEL, the interior-row kernel: "cell" runs
 * one cell per thread for every storage type instead of the paired kernel of
 * the 2-byte forms; "vec8" / "vec4" run eight / four cells per thread with
 * 128- / 64-bit population vectors (2-byte forms, rows of a multiple of eight
 * cells); "vec2" two cells per thread with packed 32-bit population words
 * (2-byte forms, rows of even length).  All give the same results. */
int plbgpu_create(int device, plbgpu_ctx** out);
int plbgpu_destroy(plbgpu_ctx* ctx);
/* Message of the last failing call on this context ("" if none). */
const char* plbgpu_last_error(const plbgpu_ctx* ctx);
/* Number of kernels this context has launched so far. */
int plbgpu_launch_count(const plbgpu_ctx* ctx, unsigned long long* count);
/* The CUDA stream (cudaStream_t) all work of the context is issued on. */
int plbgpu_get_stream(const plbgpu_ctx* ctx, void** stream);
/* Measured rate of the GPU's FP64 pipe in adds + multiplies per second
 * (independent DMUL/DADD chains on every SM, fastest of three launches).
 * The FP64 step rounds every add and multiply of the reference's collision
 * separately, so this rate, not HBM bandwidth, bounds it.  A measurement
 * aid with no counterpart in the reference. */
int plbgpu_measure_fp64_rate(plbgpu_ctx* ctx, double* ops_per_second);
/* Wait for the context's work.  Also reports (once, then clears) a diverged
 * state of any domain: PLBGPU_ERR_STATE when a step that gathered statistics
 * met a NaN or an infinity in a cell's density or kinetic energy.
 * plbgpu_receive and plbgpu_get_stats report it the same way; the domain stays
 * usable (send a new state to continue). */
int plbgpu_synchronize(plbgpu_ctx* ctx);

/* ------------------------------------------------------------ domains */

/* Allocate a domain of nx*ny*nz cells (all BGK, non-periodic, omega 1).
 * Replaces MultiBlockLattice3D construction (multiBlock/multiBlockLattice3D.hh:60-87)
 * together with CoProcessor3D::addDomain (coProcessors/coProcessor3D.h:75). */
int plbgpu_add_domain(plbgpu_ctx* ctx, int nx, int ny, int nz, int precision, int* handle);
int plbgpu_remove_domain(plbgpu_ctx* ctx, int handle);
int plbgpu_domain_info(plbgpu_ctx* ctx, int handle, int* nx, int* ny, int* nz, int* precision,
                       unsigned long long* device_bytes);

/* Periodicity per axis (PeriodicitySwitch3D::toggle, multiBlock/multiBlock3D.h:167-168). */
int plbgpu_set_periodicity(plbgpu_ctx* ctx, int handle, int px, int py, int pz);

/* omega of every BGK-family dynamics, rho0 of IncBGKdynamics (its invRho0 =
 * 1/rho0, isoThermalDynamics.hh:1353-1356), and the rho given to the
 * BounceBack / MomentumExchangeBounceBack constructors (core/dynamics.h:574). */
int plbgpu_set_params(plbgpu_ctx* ctx, int handle, double omega, double rho0, double bb_rho);

/* defineDynamics(lattice, box, dynamics) for a whole box
 * (dataProcessors/dataInitializerWrapper3D.h:170-171), and the per-cell
 * form for an arbitrary mask (`kinds` has one byte per cell of the box,
 * z fastest).  Face kinds set this way are the wrapped boundary conditions of
 * createLocalBoundaryCondition3D / createZouHeBoundaryCondition3D
 * (boundaryCondition/boundaryCondition3D.hh:1163-1167, zouHeBoundary3D.hh:338-342). */
int plbgpu_define_dynamics(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                           int kind);
int plbgpu_set_kinds(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                     const uint8_t* kinds, size_t n);
int plbgpu_get_kinds(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                     uint8_t* kinds, size_t n);

/* OnLatticeBoundaryCondition3D::setVelocityConditionOnBlockBoundaries(lattice,
 * box) of createLocalBoundaryCondition3D (boundaryCondition3D.hh:65-163): the
 * box's six faces become regularized velocity faces, its twelve edges and
 * eight corners the external velocity edges and corners above; every extent
 * of the box must be at least 3.  Edge and corner cells need their inward
 * neighbours inside the domain; a layout that breaks this is reported by the
 * next plbgpu_initialize / plbgpu_collide_and_stream as PLBGPU_ERR_ARG. */
int plbgpu_set_velocity_condition_on_block_boundaries(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0,
                                                      int y1, int z0, int z1);

/* bc->addVelocityBoundary{d}{N|P}(box, lattice), addPressureBoundary{d}{N|P},
 * addExternalVelocityEdge{plane}{N|P}{N|P} and addExternalVelocityCorner
 * {N|P}{N|P}{N|P} of the local regularized and Zou/He conditions
 * (boundaryCondition/boundaryCondition3D.h:58-140, boundaryInstantiator3D.h):
 * the face, edge or corner `kind` over the box, as plbgpu_define_dynamics,
 * plus the data-processor record the reference integrates with it (see
 * plbgpu_add_processor).  plbgpu_set_velocity_condition_on_block_boundaries
 * records its 26 processors the same way, in the reference's order. */
int plbgpu_add_boundary(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1, int kind);

/* The lattice's data-processor list, which every saved lattice state's
 * description carries (io/multiBlockWriter3D.cpp:113-136: name, domain,
 * serialized data, level, block ids, indexed by place in the list).  The
 * GPU's own boundary handling follows the cell kinds; the list is what the
 * reference lattice built by the same calls would hold.  In `name`, "%TD"
 * stands for "double_<Descriptor>" of the saved lattice, as the reference
 * names generators after their template arguments
 * ("OuterVelocityEdge_%TD_0_-1_1").  plbgpu_load_processors appends the
 * processors listed in a description that meet the domain, clipped to it,
 * as readXmlProcessors does for a loaded block
 * (io/multiBlockReader3D.cpp:91-133).  plbgpu_get_processor fails when a
 * buffer is too small; nblocks receives the block count either way. */
int plbgpu_add_processor(plbgpu_ctx* ctx, int handle, const char* name, const long long* domain6,
                         const char* data, long long level, const long long* blocks, int nblocks);
int plbgpu_clear_processors(plbgpu_ctx* ctx, int handle);
int plbgpu_processor_count(plbgpu_ctx* ctx, int handle, int* count);
int plbgpu_get_processor(plbgpu_ctx* ctx, int handle, int index, char* name, size_t name_cap, long long* domain6,
                         char* data, size_t data_cap, long long* level, long long* blocks, int blocks_cap,
                         int* nblocks);
int plbgpu_load_processors(plbgpu_ctx* ctx, int handle, const char* plb_path);

/* Sparse domain: computeSparseManagement(field) (offLattice/makeSparse3D.hh:
 * 107-160) over the regular distribution createRegularDistribution3D(nx, ny,
 * nz, bx, by, bz) (multiBlock/staticRepartitions3D.cpp:38-63).  A block is
 * kept when any cell of it has a non-zero value in `field` (n = nx*ny*nz
 * int32, z fastest); the cells of the other blocks leave the lattice: they are
 * never updated, read back as zeros, count in no reduction or statistic, and
 * their neighbours treat them like the outside of a non-periodic domain (the
 * domain-edge rule).  keep (optional, bx*by*bz entries, x-major) receives the
 * selection.  Steps on a sparse domain go by 32-cell row tiles, rebuilt when
 * the kinds or the periodicity change: tiles whose neighbourhood lies in the
 * lattice take the interior-row kernels, the other tiles of interior rows the
 * one-cell row kernel with per-cell masks of the neighbours outside the
 * lattice, the tiles of border rows the general addressing; tiles without a
 * live cell are not stepped. */
int plbgpu_select_sparse_blocks(plbgpu_ctx* ctx, int handle, const int32_t* field, size_t n, int bx, int by,
                                int bz, uint8_t* keep, size_t nblocks);

/* setBoundaryVelocity / setBoundaryDensity (dataInitializerWrapper3D.h:99-118),
 * constant over a box or one value per cell of the box (`values`: 3 doubles
 * per cell for velocity, 1 per cell for density). */
int plbgpu_set_boundary_velocity(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0,
                                 int z1, double ux, double uy, double uz);
int plbgpu_set_boundary_velocity_field(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1,
                                       int z0, int z1, const double* values, size_t n);
int plbgpu_set_boundary_density(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0,
                                int z1, double rho);
int plbgpu_set_boundary_density_field(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1,
                                      int z0, int z1, const double* values, size_t n);

/* setExternalVector(lattice, box, forceBeginsAt, F) for the Guo force
 * (dataInitializerWrapper3D.h:154-155), constant or per cell (3 doubles). */
int plbgpu_set_force(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                     double fx, double fy, double fz);
int plbgpu_set_force_field(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                           const double* values, size_t n);

/* initializeMomentumExchange(lattice, boundingBox)
 * (boundaryCondition/bounceBackModels3D.hh:248-271): record, for every
 * momentum-exchange cell, the directions pointing to fluid. */
int plbgpu_initialize_momentum_exchange(plbgpu_ctx* ctx, int handle);

/* initializeAtEquilibrium(lattice, box, rho, u) (dataInitializerWrapper3D.h:122-123,
 * core/cell.hh iniCellAtEquilibrium), constant or per cell (`rho_u`: 4 doubles
 * per cell: rho, ux, uy, uz). */
int plbgpu_initialize_at_equilibrium(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0,
                                     int z1, double rho, double ux, double uy, double uz);
int plbgpu_initialize_at_equilibrium_field(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1,
                                           int z0, int z1, const double* rho_u, size_t n);

/* lattice.initialize() (multiBlock/multiBlock3D.cpp:330-332): run the
 * boundary-face completion once on the current state. */
int plbgpu_initialize(plbgpu_ctx* ctx, int handle);

/* ------------------------------------------------------------ transfer */

/* Host -> device / device -> host of the populations of a sub-box, FP64
 * f-bar, transfer layout above; n = number of doubles in buf (19 per cell).
 * CoProcessor3D::send / receive (coProcessors/coProcessor3D.h:80-96).
 * buf may be host memory (pageable or pinned) or device memory.  When the GPU
 * can address buf -- device, managed or pinned memory, or pageable memory on
 * a GPU that uses the host's page tables (GB300 with its Grace CPU) -- one
 * kernel reads or writes it directly, coalesced; otherwise the records go
 * through a device staging buffer of at most 64 MiB, chunk by chunk
 * (environment variable PLBGPU_STAGED_TRANSFERS=1 at plbgpu_create forces
 * this path).  Both calls return once buf may be reused. */
int plbgpu_send(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                const double* buf, size_t n);
int plbgpu_receive(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                   double* buf, size_t n);
/* The same with FP32 records (19 floats per cell): the transfer of a
 * single-precision lattice, CoProcessor3D<float>::send / receive. */
int plbgpu_send_f32(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                    const float* buf, size_t n);
int plbgpu_receive_f32(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                       float* buf, size_t n);

/* ------------------------------------------------------------ time stepping */

/* nsteps collide-and-stream steps of the whole domain: collision, streaming,
 * boundary-face completion, periodic wrap -- the full
 * MultiBlockLattice3D::collideAndStream() (multiBlock/multiBlockLattice3D.hh:318-357)
 * including executeInternalProcessors and the envelope update.  When
 * collect_stats is non-zero the internal statistics (average rho-bar,
 * average u^2, max u^2, momentum-exchange force) are gathered during the last
 * of the nsteps steps.  Asynchronous: returns once the work is queued. */
int plbgpu_collide_and_stream(plbgpu_ctx* ctx, int handle, int nsteps, int collect_stats);

/* The co-processor cycle transferToCoProcessors -> nsteps x collideAndStream
 * -> transferFromCoProcessors (coProcessors/coProcessorCommunication3D.hh:
 * 34-70, multiBlock/multiBlockLattice3D.hh:318-357) in one call: the whole
 * domain's records `in` (n = 19 per cell, the plbgpu_send layout) are sent,
 * nsteps steps run, and the state is received into `out` (which may be `in`).
 * With stats_every > 0 the statistics of every stats_every-th step and of the
 * last step are written to `stats`, 7 doubles each in the plbgpu_get_stats
 * layout (ceil(nsteps / stats_every) records, nstats doubles available).  The
 * result is bit for bit that of plbgpu_send, plbgpu_collide_and_stream and
 * plbgpu_receive.  When the GPU addresses both buffers directly (device or
 * pinned memory, or any host memory on a GB300), the domain has no edges,
 * corners or dropped blocks and its form is not PLBGPU_BF16_SR (whose random
 * rounding bits depend on the kernel that stores a slot), the transfers
 * overlap the steps: the domain is cut into x-slabs moved by a copy kernel
 * on a few SMs through a ring of four slab-sized staging slots; slab j takes
 * its first step once its records are in and step s once slabs j - 1 .. j + 1
 * took step s - 1, so the first steps run as a ramp behind the send, and the
 * last steps as a ramp that finishes slab 0 first, each slab received while
 * the later ones step. */
int plbgpu_run_host(plbgpu_ctx* ctx, int handle, const double* in, double* out, size_t n, int nsteps,
                    int stats_every, double* stats, size_t nstats);

/* The order of the operations of plbgpu_run_host's overlapped path for a
 * domain of nx >= 4 x-planes (periodic_x non-zero: periodic along x), nsteps
 * >= 2 steps, statistics every stats_every steps and storage form
 * `precision`.  Host logic only (no context, no GPU).  Slab j holds the planes
 * j * slab_width .. min(nx, (j + 1) * slab_width) - 1.  *count = the number of
 * operations; with ops non-null (cap >= 3 * count ints) each is written as
 * (kind, slab, step): kind 0 = slab sent (its records copied in and
 * inserted), 1 = step `step` of the slab, 2 = slab received after the last
 * step, 3 = the steps [slab, step) of the whole domain. */
int plbgpu_run_host_plan(int nx, int periodic_x, int nsteps, int stats_every, int precision, int* slab_width,
                         int* ops, size_t cap, size_t* count);

/* Statistics of the last step that gathered them (BlockStatistics::evaluate,
 * core/blockStatistics.cpp:77-110; MultiBlock3D::getInternalStatistics):
 * out[0] average rho-bar, out[1] average u^2, out[2] max u^2,
 * out[3..5] sum of -momentum exchange (drag on the obstacle) x,y,z,
 * out[6] number of cells that gathered statistics. */
int plbgpu_get_stats(plbgpu_ctx* ctx, int handle, double out[7]);

/* computeAverageEnergy / computeAverageDensity over a box
 * (dataProcessors/dataAnalysisWrapper3D.hh:1226-1262). */
int plbgpu_reduce(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                  double* avg_energy, double* avg_density);

/* computeVelocity / computeDensity (dataProcessors/dataAnalysisWrapper3D.h:80-132):
 * the velocity (3 doubles per cell) or density (1 per cell) each cell's
 * dynamics reports, over a box, in the transfer order (z fastest). */
int plbgpu_compute_velocity(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                            double* out, size_t n);
int plbgpu_compute_density(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                           double* out, size_t n);

/* Run nsteps steps and time them with CUDA events recorded on the context's
 * stream (milliseconds). */
int plbgpu_time_steps(plbgpu_ctx* ctx, int handle, int nsteps, int collect_stats, float* ms);

/* ------------------------------------------------------------ external rho-bar / j */

/* A domain's external moment fields: rho-bar and j (4 values per cell),
 * FP64 for the FP64 form and FP32 otherwise -- the MultiScalarField3D /
 * MultiTensorField3D<T,3> pair the reference passes to its processors.
 * plbgpu_compute_rhobar_j fills them with BoxRhoBarJfunctional3D over the
 * whole domain (each cell's computeRhoBarJ, dataAnalysisFunctional3D.hh:528-549);
 * set/get move a box of (rho-bar, jx, jy, jz) per cell, z fastest. */
int plbgpu_compute_rhobar_j(plbgpu_ctx* ctx, int handle);
int plbgpu_set_rhobar_j(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                        const double* values, size_t n);
int plbgpu_get_rhobar_j(plbgpu_ctx* ctx, int handle, int x0, int x1, int y0, int y1, int z0, int z1,
                        double* out, size_t n);

/* nsteps steps of ExternalRhoJcollideAndStream3D (basicDynamics/dynamicsProcessor3D.hh:
 * 41-200): each cell's collideExternal with rho-bar and j from the fields
 * instead of its own moments, then streaming, the face completion and the
 * edge / corner processors.  With recompute non-zero, BoxRhoBarJfunctional3D
 * refreshes the fields from the streamed populations after every step, before
 * the boundary processors -- the order of a lattice that integrates the two
 * processors at levels 0 and 3 and is advanced by executeInternalProcessors().
 * The BGK-family collisions gather no statistics in this form; the momentum
 * exchange still does.  PLBGPU_ERR_STATE when the fields were never set. */
int plbgpu_collide_and_stream_external(plbgpu_ctx* ctx, int handle, int nsteps, int recompute,
                                       int collect_stats);

/* ------------------------------------------------------------ checkpoints */

/* Block kinds of saveBinaryBlock / loadBinaryBlock (io/serializerIO_3D.cpp:37-66):
 * the values per cell are the ones Block3D serialization writes -- the 19
 * populations (f-bar) and, for the forced descriptor, the 3 force components
 * after them (core/cell.hh:103-110); computeDensity / computeVelocity fields;
 * the external rho-bar / j fields. */
#define PLBGPU_BLOCK_LATTICE 0          /* D3Q19 lattice: 19 doubles per cell */
#define PLBGPU_BLOCK_FORCED_LATTICE 1   /* ForcedD3Q19 lattice: 19 + 3 doubles per cell */
#define PLBGPU_BLOCK_DENSITY 2          /* computeDensity field: 1 double per cell (save only) */
#define PLBGPU_BLOCK_VELOCITY 3         /* computeVelocity field: 3 doubles per cell (save only) */
#define PLBGPU_BLOCK_RHOBAR 4           /* external rho-bar field: 1 double per cell */
#define PLBGPU_BLOCK_J 5                /* external j field: 3 doubles per cell */

/* saveBinaryBlock(block, path, enforce_uint) / loadBinaryBlock: the file is
 * base64 text -- the byte count (8 bytes, or 4 with enforce_uint), then the
 * cell records x-major, z fastest, as the reference's default stream ordering
 * writes them (io/serializerIO.cpp:64-115, multiBlock/multiBlockSerializer3D.cpp:
 * 61-129).  The records are assembled and encoded (decoded) on the device in
 * slabs of whole x-planes; only the text crosses to the host.  A file whose
 * byte count does not match the domain, or that is not base64, is refused
 * (PLBGPU_ERR_ARG). */
int plbgpu_save_binary_block(plbgpu_ctx* ctx, int handle, int what, const char* path, int enforce_uint);
int plbgpu_load_binary_block(plbgpu_ctx* ctx, int handle, int what, const char* path, int enforce_uint);

/* parallelIO::save(block, base, false) / parallelIO::load(plb, block, false)
 * -- the files of saveState / loadState (io/utilIO_3D.cpp:45-75,
 * io/multiBlockWriter3D.cpp:53-137, 201-213, io/multiBlockReader3D.cpp:135-270):
 * <base>.dat holds the raw cell records of each component (x-major, z
 * fastest, no header) and <base>.plb their XML description (block family,
 * descriptor, cell size, bounding box, components, byte offsets, data file).
 * Save writes one component, the whole domain; load accepts any number of
 * components (the reference writes one per block) with a bounding box of the
 * domain's size.  Loading a lattice state saved with dynamic content takes its
 * populations (and force) only, as load(plb, block, false) does; a field's
 * records are the same with or without dynamic content. */
int plbgpu_save_state(plbgpu_ctx* ctx, int handle, int what, const char* base);
int plbgpu_load_state(plbgpu_ctx* ctx, int handle, int what, const char* plb_path);

/* parallelIO::save(lattice, base, true) / parallelIO::load(plb, lattice, true)
 * -- the states with dynamic content, parallelIO::save's default
 * (io/multiBlockWriter3D.h:42-43, atomicBlock/blockLattice3D.hh:703-722,
 * 812-845): in front of every cell's static values, its serialized dynamics
 * chain (class id, then the parameters: omega, 1/rho0 of incompressible BGK,
 * the wall density, the momentum-exchange fluid directions, a face's stored
 * velocity or rho-bar around its BGK base), and in <base>.plb a DynamicsDict
 * mapping the ids to the dynamics names.  what: PLBGPU_BLOCK_LATTICE or
 * PLBGPU_BLOCK_FORCED_LATTICE.  Save writes one component (cells outside the
 * lattice of a sparse domain as NoDynamics with zero populations, which a
 * reference lattice on the same sparse blocks does not have and skips).  Load
 * reads any number of components that cover every cell of the lattice (cells
 * outside it stay outside, as the reference's load fills only the blocks that
 * exist), then sets the cell kinds, the boundary values, the
 * momentum-exchange directions, omega / rho0 / the wall density, and the
 * populations, as the reference regenerates the dynamics objects.  A state
 * whose cells need more than the domain holds -- dynamics without a GPU kind,
 * several omegas, rho0s or wall densities, a stored-velocity cell off the
 * domain's edges and corners -- is refused (PLBGPU_ERR_ARG) before anything
 * changes.  Both lattice saves write the domain's data-processor list
 * (plbgpu_add_processor) into the description; the loads leave the domain's
 * list as it is, as the reference's load copies cells only
 * (io/multiBlockReader3D.cpp:261-268) -- plbgpu_load_processors reads it. */
int plbgpu_save_state_dynamic(plbgpu_ctx* ctx, int handle, int what, const char* base);
int plbgpu_load_state_dynamic(plbgpu_ctx* ctx, int handle, int what, const char* plb_path);

/* ------------------------------------------------------------ voxelizer */

/* Voxel flags of a closed triangle mesh on the box [0, nx-1] x [0, ny-1] x
 * [0, nz-1], as voxelize(mesh, domain, borderWidth) gives them
 * (offLattice/voxelizer.hh:106-141, DetectBorderLineFunctional3D :653-685):
 * 1 outside, 2 outerBorder (outside with an inside cell within border_width),
 * 3 inside, 4 innerBorder.  The box's outer layer is outside.  triangles:
 * n_triangles x 3 vertices x (x, y, z) in lattice units, each triangle's
 * normal (v1 - v0) x (v2 - v0) pointing out of the body (a cell centre on the
 * surface counts as inside).  flags: n = nx*ny*nz int32, z fastest.  A lattice
 * line crossing the surface more than 64 times is refused (PLBGPU_ERR_ARG).
 * The surface must lie inside the box's outer layer, which the reference
 * seeds as outside: a body cut by that layer has no path-independent answer. */
int plbgpu_voxelize(plbgpu_ctx* ctx, const double* triangles, size_t n_triangles, int nx, int ny, int nz,
                    int border_width, int32_t* flags, size_t n);

/* ------------------------------------------------------------ adjoint */

/* Discrete adjoint of the collide-and-stream step (no counterpart in the
 * reference), for domains of BGK, Guo, incompressible BGK, bounce-back,
 * momentum-exchange bounce-back, no-dynamics, regularized or Zou/He velocity
 * and pressure face cells, and the external velocity edges and corners
 * (their finite-difference processors replayed after each step and
 * reversed; an edge or corner next to a Guo-forced cell is refused).  Face,
 * edge and corner cells count as zero velocity in the velocity objectives.
 * The objective is J = 1/2 sum over cells |u(T) - u*|^2
 * with u the velocity each cell's dynamics reports (computeVelocity,
 * dataProcessors/dataAnalysisWrapper3D.h:127-132).
 *
 * plbgpu_adjoint_forward: run T steps from the current state, keeping a
 * checkpoint every K steps (K divides T); the domain ends at step T.  K = 0
 * picks the smallest divisor of T whose checkpoints fit in 80% of the free
 * device memory (K = 1 keeps every state and the backward sweep recomputes
 * nothing); plbgpu_adjoint_interval reports the K of the recorded run.
 * plbgpu_adjoint_backward: J, dJ/dF per cell (3 doubles per cell, transfer
 * order; may be NULL) and dJ/domega for that run, recomputing each segment
 * of K steps from its checkpoint; `ms` (may be NULL) receives the device time
 * of the backward sweep, recomputation included.
 * plbgpu_tangent_linear (FP64 domains): J and the directional derivative
 * dJ = grad J . (dforce, domega) from a dual-number run of T steps from the
 * current state, which it leaves unchanged.
 *
 * The _weighted forms take the objective J = sum over cells w . u(T) instead
 * (w: 3 doubles per cell, transfer order), e.g. the mean flux
 * w = (1/n, 0, 0) from which a permeability follows.
 * plbgpu_adjoint_steady_weighted: the same gradients at a steady state (the
 * domain's current state, taken as converged): `iterations` reverse steps
 * linearised around that one state, no recorded run and no checkpoints
 * (three states of memory); the gradient converges as the flow would relax.
 *
 * The _drag forms take J = direction . D with D the momentum-exchange drag
 * of the state (what the next collision records on MomentumExchangeBounceBack
 * cells, bounceBackModels.hh:100-136; needs plbgpu_initialize_momentum_exchange). */
int plbgpu_adjoint_forward(plbgpu_ctx* ctx, int handle, int T, int K);
int plbgpu_adjoint_interval(plbgpu_ctx* ctx, int handle, int* K);
int plbgpu_adjoint_backward(plbgpu_ctx* ctx, int handle, const double* u_target, size_t n_target,
                            double* objective, double* grad_force, size_t n_grad, double* grad_omega,
                            float* ms);
int plbgpu_tangent_linear(plbgpu_ctx* ctx, int handle, int T, const double* dforce, size_t n_dforce,
                          double domega, const double* u_target, size_t n_target, double* objective,
                          double* directional);
int plbgpu_adjoint_backward_weighted(plbgpu_ctx* ctx, int handle, const double* weights, size_t n_weights,
                                     double* objective, double* grad_force, size_t n_grad, double* grad_omega,
                                     float* ms);
int plbgpu_tangent_linear_weighted(plbgpu_ctx* ctx, int handle, int T, const double* dforce, size_t n_dforce,
                                   double domega, const double* weights, size_t n_weights, double* objective,
                                   double* directional);
int plbgpu_adjoint_steady_weighted(plbgpu_ctx* ctx, int handle, int iterations, const double* weights,
                                   size_t n_weights, double* objective, double* grad_force, size_t n_grad,
                                   double* grad_omega, float* ms);
int plbgpu_adjoint_backward_drag(plbgpu_ctx* ctx, int handle, const double* direction, double* objective,
                                 double* grad_force, size_t n_grad, double* grad_omega, float* ms);
int plbgpu_tangent_linear_drag(plbgpu_ctx* ctx, int handle, int T, const double* dforce, size_t n_dforce,
                               double domega, const double* direction, double* objective, double* directional);
int plbgpu_adjoint_steady_drag(plbgpu_ctx* ctx, int handle, int iterations, const double* direction,
                               double* objective, double* grad_force, size_t n_grad, double* grad_omega, float* ms);

/* ------------------------------------------------------------ co-processor form */

/* The four calls of plb::CoProcessor3D<double> (coProcessors/coProcessor3D.h:41-116)
 * with its return convention: 1 = success, 0 = failure.  A domain created
 * by plbgpu_cp_add_domain is all BGK with the given omega, non-periodic,
 * FP64, exactly like D3Q19ExampleCoProcessor3D (coProcessor3D.hh:36-76);
 * `data` holds 19 doubles per cell of the sub-box, so nbytes = 152 * cells. */
int plbgpu_cp_add_domain(plbgpu_ctx* ctx, long nx, long ny, long nz, double omega, int* handle);
int plbgpu_cp_send(plbgpu_ctx* ctx, int handle, long x0, long x1, long y0, long y1, long z0, long z1,
                   const char* data, size_t nbytes);
int plbgpu_cp_receive(plbgpu_ctx* ctx, int handle, long x0, long x1, long y0, long y1, long z0, long z1,
                      char* data, size_t nbytes);
int plbgpu_cp_collide_and_stream(plbgpu_ctx* ctx, int handle);
/* plb::CoProcessor3D<float> (the reference's single-precision lattice,
 * e.g. jlabos/src/testing/test_cylinder.py:96-97): an FP32 domain (FP32
 * arithmetic and storage) whose `data` holds 19 floats per cell, nbytes =
 * 76 * cells.  collideAndStream is plbgpu_cp_collide_and_stream. */
int plbgpu_cp_add_domain_f32(plbgpu_ctx* ctx, long nx, long ny, long nz, double omega, int* handle);
int plbgpu_cp_send_f32(plbgpu_ctx* ctx, int handle, long x0, long x1, long y0, long y1, long z0, long z1,
                       const char* data, size_t nbytes);
int plbgpu_cp_receive_f32(plbgpu_ctx* ctx, int handle, long x0, long x1, long y0, long y1, long z0, long z1,
                          char* data, size_t nbytes);

/* ------------------------------------------------------------ allocation-free form */

/* Rows of scratch available to plbgpu_reduce_noalloc: nx * ny may not exceed it. */
#define PLBGPU_NOALLOC_MAX_ROWS 262144

/* Average energy and density of a lattice held in caller-owned device memory,
 * computed without allocating any device memory.  No counterpart in the
 * reference: it serves callers that cannot call cudaMalloc (applications with
 * their own device-memory pool or a fixed budget, hosts where the runtime
 * allocator is off limits).
 *
 * populations: 19 planes of FP64 f-bar, plane i at populations + i * stride,
 *              cell (x, y, z) at index (x * ny + y) * nz + z, post-stream
 *              (natural) order -- device memory.
 * kinds:       one byte per cell (PLBGPU_BGK, PLBGPU_INCBGK, PLBGPU_BOUNCEBACK,
 *              PLBGPU_MOMENTUM_EXCHANGE, PLBGPU_NODYNAMICS) -- device memory.
 *              Any other kind makes both results NaN.
 * result:      device memory for 2 doubles: average energy, average density.
 * stream:      cudaStream_t the two kernels are queued on (NULL = default).
 *
 * The scratch is a 4 MiB array of PLBGPU_NOALLOC_MAX_ROWS row sums in the
 * library's device image, kept by every GPU that loads the library until the
 * process exits.  Sizes with nx * ny > PLBGPU_NOALLOC_MAX_ROWS are rejected
 * with PLBGPU_ERR_ARG.  All calls share the array; calls whose kernels overlap
 * on the GPU race on it.  The first call on a device looks up the array's
 * address with that device current: make it before any stream capture.  The
 * address is kept for the life of the process, so after a cudaDeviceReset of
 * that device this entry point must not be called again.
 * Asynchronous: returns once both kernels are queued. */
int plbgpu_reduce_noalloc(const double* populations, long long stride, const uint8_t* kinds, int nx, int ny,
                          int nz, double bb_rho, double rho0, double* result, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PLBGPU_H */
