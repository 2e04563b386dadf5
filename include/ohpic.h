/*
 * ohpic.h -- C ABI of the GB300 particle hot path for ohhelppic3d.
 *
 * The reference (Nkzono99/ohhelppic3d, Fortran 2008) advances particles one
 * record at a time through polymorphic type-bound procedures:
 *
 *   t_Scatter%scatter(particle, ohfield, amount, ps)       src/scatter/scatter.f90:15-24
 *   t_FieldSolver%solve(rho, aj, eb, phi, ohhelp)          src/field_solver/field_solver.f90:15-25
 *   t_Interpolator%interp(particle, field, ps) -> ret(6)   src/interpolator/interpolator.f90:16-25
 *   t_ParticleMover%move(particle, qm, eb, dt)             src/particle_mover/particle_mover.f90:16-24
 *   t_ParticleBoundary%apply(particle, dt)                 src/particle_boundary/particle_boundary.f90:14-20
 *
 * called from the loops of mainstep (src/ohhelppic3d.f90:311-358).  A call per
 * particle across a language boundary cannot feed a GPU, so this ABI offers the
 * same operations batched over every particle of the run, with the particles
 * and fields resident in device memory between calls.  The Fortran side binds
 * these functions with ISO_C_BINDING interfaces whose derived types mirror the
 * structs below field by field.
 *
 * Conventions
 *   - Every function returns an int status: OHPIC_OK (0) or an OHPIC_ERR_* code.
 *     No C++ exception crosses the ABI.  ohpic_last_error() gives the message.
 *   - Host arrays are borrowed for the duration of the call only.
 *   - Work is ordered on the context's own CUDA stream.  Calls that return host
 *     data (download, diagnostics) synchronise that stream; the others do not.
 *   - One context belongs to one host thread at a time.
 *   - Fields are exchanged as nx*ny*nz doubles with x fastest, which is the
 *     interior of the reference's t_OhField%values(1, 0:nx-1, 0:ny-1, 0:nz-1, 1)
 *     (src/ohhelp/ohfield.f90:54,165-169); ohpic_download_field_ohfield() fills
 *     the full layout including halos.
 */
#ifndef OHPIC_H
#define OHPIC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OHPIC_MAX_SPECIES 8
#define OHPIC_ABI_VERSION 1

/* Status codes. */
enum {
    OHPIC_OK = 0,
    OHPIC_ERR_INVALID = 1,      /* bad argument or configuration */
    OHPIC_ERR_OOM = 2,          /* device or pinned-host allocation failed */
    OHPIC_ERR_CUDA = 3,         /* a CUDA / cuFFT call failed */
    OHPIC_ERR_BOUNDS = 4,       /* a kernel saw an index outside its grid (device error flag) */
    OHPIC_ERR_TIMEOUT = 5,      /* a bounded device wait ran out */
    OHPIC_ERR_CAPACITY = 6,     /* more particles than the species capacity */
    OHPIC_ERR_UNSUPPORTED = 7,  /* the reference's per-particle entry points (see below) */
    OHPIC_ERR_NONFINITE = 8,    /* NaN or Inf in the particle state */
    OHPIC_ERR_REJECTED = 9      /* serving: request does not fit the memory budget */
};

/* Precision forms. */
enum {
    OHPIC_FP64 = 0,  /* plain form: absolute FP64 positions and velocities */
    OHPIC_FP32 = 1   /* precision form: int32 cell + FP32 in-cell offset, FP32 velocity */
};

/* CIC weight convention.  The reference gives node floor(x) the weight
 * r = x - floor(x) and node floor(x)+1 the weight 1-r
 * (src/interpolator/linear_interpolator.f90:54-64, src/scatter/linear_scatter.f90:41-52);
 * OHPIC_WEIGHTS_STANDARD is the textbook assignment (1-r, r). */
enum { OHPIC_WEIGHTS_REFERENCE = 0, OHPIC_WEIGHTS_STANDARD = 1 };

/* Field selectors. */
enum { OHPIC_RHO = 0, OHPIC_PHI = 1, OHPIC_EX = 2, OHPIC_EY = 3, OHPIC_EZ = 4 };

typedef struct ohpic_config {
    int32_t nx, ny, nz;         /* periodic grid, dx = 1 (parameters.f90:209-211) */
    int32_t nspecies;           /* 1..OHPIC_MAX_SPECIES (parameters.f90:239) */
    int32_t precision;          /* OHPIC_FP64 or OHPIC_FP32 */
    int32_t weights;            /* OHPIC_WEIGHTS_* */
    int32_t sort_every;         /* cell sort cadence in steps; 0 = only explicit ohpic_sort */
    int32_t tile[3];            /* tile shape in cells; 0 = tuned default */
    int32_t track_ids;          /* 1: keep a per-particle id through sorts */
    int32_t device;             /* CUDA device ordinal */
    double dt;                  /* default time step (parameters.f90:213) */
    double b0[3];               /* uniform magnetic field passed to Boris */
    double qm[OHPIC_MAX_SPECIES];   /* charge-to-mass ratio (parameters.f90:240) */
    double q[OHPIC_MAX_SPECIES];    /* charge per macro-particle (parameters.f90:259-260) */
    int64_t capacity[OHPIC_MAX_SPECIES]; /* maximum particles per species */
} ohpic_config;

typedef struct ohpic_diag {
    int64_t count[OHPIC_MAX_SPECIES];
    int64_t crossings[3];       /* particles that wrapped along x, y, z in the last push */
    int64_t outside_tile;       /* particles the last push served from global memory */
    int64_t step;               /* pushes since creation */
    double total_charge;        /* sum of rho over nodes (FP64 reduction) */
    double field_energy;        /* 0.5 * sum |E|^2 over nodes */
    double kinetic_energy;      /* sum 0.5 * (q/qm) |v|^2 over particles */
    double momentum[3];         /* sum (q/qm) v */
} ohpic_diag;

/* Injector parameters of one species (src/particle_injector/particle_injector_manager.f90:55-70
 * with the Maxwellian enabled, sigma = vth). */
typedef struct ohpic_species_init {
    double ppc;                 /* macro-particles per cell inside the range */
    double vth;                 /* Maxwellian standard deviation; clipped at +-6 vth */
    double drift[3];            /* added after the clip (beams) */
    double lo[3], hi[3];        /* position range, clipped to [0, n] */
} ohpic_species_init;

typedef struct ohpic_ctx ohpic_ctx;

/* Fills cfg with defaults (FP64 form, reference weights, sort every 20 steps,
 * tuned tiles, ids tracked, device 0).  Grid, species and dt stay zero. */
void ohpic_config_default(ohpic_config *cfg);

/* Creates a context that owns all device memory and one CUDA stream.
 * Replaces the set-up of src/ohhelppic3d.f90:114-122 (field allocation),
 * :195 (new_LinearScatter), :261-269 (new_PoissonFieldSolver), :273
 * (new_LinearInterpolator) and :279-282 (mover factory and boundaries). */
int ohpic_create(const ohpic_config *cfg, ohpic_ctx **out);
int ohpic_destroy(ohpic_ctx *ctx);

/* Particle transfer.  The AoS form reads records of stride_bytes whose first
 * six doubles are x, y, z, vx, vy, vz, i.e. the leading members of the
 * reference's oh_particle (src/ohhelp/ohparticles.f90:17, used by
 * particle_injector_with_distribution.f90:196-201).  Upload replaces the
 * species' particles; n may be 0.  The FP32 form refuses positions it cannot
 * wrap into the grid (OHPIC_ERR_BOUNDS) and positions or velocities that are
 * not finite in FP32 (OHPIC_ERR_NONFINITE); a refused upload leaves the
 * species empty. */
int ohpic_upload_particles(ohpic_ctx *ctx, int species, const void *pbuf, int64_t n,
                           int64_t stride_bytes);
int ohpic_upload_particles_soa(ohpic_ctx *ctx, int species, const double *x, const double *y,
                               const double *z, const double *vx, const double *vy,
                               const double *vz, int64_t n);
/* Device-side initial conditions with the reference injector's random streams:
 * PCG32 seeded (initstate, initseq) and advanced by `advance`
 * (src/ohhelppic3d.f90:111-112), then per species one random_fix draw
 * (src/radom/random_generator.f90:45-58) and 7 draws per particle (x, y, z,
 * then the 4-draw Maxwellian; particle_injector_with_distribution.f90:51-69).
 * Positions are bit-identical to the reference injector fed the same streams;
 * velocities use the device libm.  counts_out (nullable) receives the
 * per-species counts.  Replaces initialize_particles (particle_injector_manager.f90:88-98). */
int ohpic_init_particles(ohpic_ctx *ctx, uint64_t initstate, uint64_t initseq, uint64_t advance,
                         const ohpic_species_init *species, int64_t *counts_out);

/* Download in device order; ids (nullable) receive each particle's index in
 * the last upload, so a caller can restore its own order. */
int ohpic_download_particles_soa(ohpic_ctx *ctx, int species, double *x, double *y, double *z,
                                 double *vx, double *vy, double *vz, uint32_t *ids,
                                 int64_t capacity, int64_t *n_out);
int ohpic_download_particles(ohpic_ctx *ctx, int species, void *pbuf, int64_t capacity,
                             int64_t stride_bytes, int64_t *n_out);

/* t_Scatter%scatter over every particle (linear_scatter.f90:22-55 driven by
 * ohhelppic3d.f90:311-320): rho = 0, CIC deposit of q_s, periodic fold. */
int ohpic_scatter(ohpic_ctx *ctx);

/* t_FieldSolver%solve (poisson_field_solver.f90:90-175): spectral Poisson
 * solve of rho (poisson_solver3d.f90:134-207) and E = -grad phi by the
 * staggered difference plus two-point average. */
int ohpic_solve(ohpic_ctx *ctx);

/* t_Interpolator%interp over every particle of one species: e_out receives
 * 3*n doubles (Ex, Ey, Ez per particle) in device order; capacity is the number
 * of doubles e_out holds (>= 3*n, else OHPIC_ERR_CAPACITY). */
int ohpic_interp(ohpic_ctx *ctx, int species, double *e_out, int64_t capacity, int64_t *n_out);

/* t_ParticleMover%move (Boris, particle_mover_boris.f90:21-64) followed by
 * t_ParticleBoundaries%apply twice (ohhelppic3d.f90:353,355) over every
 * particle, gathering E from the last solve.  Leaves rho stale. */
int ohpic_move(ohpic_ctx *ctx, double dt);

/* Fused gather + Boris + periodic wrap + deposit of the new positions: one
 * read and one write of each particle, after which rho holds the charge
 * the next mainstep would scatter. */
int ohpic_push(ohpic_ctx *ctx, double dt);

/* nsteps x mainstep: solve, push, and the cell sort every sort_every steps.
 * Scatters first if rho is stale. */
int ohpic_step(ohpic_ctx *ctx, double dt, int nsteps);

/* Periodic counting sort of every species by tile-major cell index (in the
 * FP32 form with ohpic_tuning.sort_lead > 0: the cell each particle reaches
 * after that many steps of straight-line motion).  In the FP32 form the sort
 * leaves each particle as a 32-byte record; the next ohpic_push/ohpic_step in
 * the default launch shape reads the records and writes the particle arrays
 * itself, and every other call that touches particles converts them first.
 * Callers see no difference but the timing and the storage order. */
int ohpic_sort(ohpic_ctx *ctx);

/* Field exchange, nx*ny*nz doubles with x fastest.  Uploading rho or E
 * replaces the device copy (for isolated tests of solve or move). */
int ohpic_download_field(ohpic_ctx *ctx, int which, double *host);
int ohpic_upload_field(ohpic_ctx *ctx, int which, const double *host);

/* Download into the reference's t_OhField%values(nelem, lo:hi, ...) layout for
 * one field slot (ohfield.f90:165-169): values has nelem leading elements per
 * node (1 for rho/phi, 6 for eb, whose elements 1-3 receive E and 4-6 B0) and
 * node ranges lo[d]..hi[d] (inclusive, may extend past the grid as halos,
 * filled periodically).  which: OHPIC_RHO, OHPIC_PHI or OHPIC_EX (whole eb). */
int ohpic_download_field_ohfield(ohpic_ctx *ctx, int which, double *values, int nelem,
                                 const int32_t lo[3], const int32_t hi[3]);

/* Checkpoint and restart of the particle state: the restart the reference's
 * [continuaus] parameters describe (parameters.f90:91-94) but never implement.
 * A snapshot is a byte image in host memory, written by the caller wherever it
 * likes: a 256-byte header, then per species the particle arrays in the
 * context's own form, bit for bit (FP32 form: packed cell, 3 offsets, 3
 * velocities, id = 32 bytes per particle; FP64 form: 6 doubles and the id =
 * 52 bytes, padded to 8).  The header holds the grid, form, species count, the
 * per-species counts and the step counters; the physics (qm, q, B0, dt) comes
 * from the restoring context's own config.  After a restore the next step
 * deposits the restored particles again, so a run continues bit-identically in
 * either form (both deposits are integer fixed point).
 * ohpic_snapshot_load() requires the same grid, form and species count, and
 * counts within the context's capacities. */
int ohpic_snapshot_size(ohpic_ctx *ctx, int64_t *bytes);
int ohpic_snapshot_save(ohpic_ctx *ctx, void *host, int64_t bytes);
int ohpic_snapshot_load(ohpic_ctx *ctx, const void *host, int64_t bytes);

int ohpic_diagnostics(ohpic_ctx *ctx, ohpic_diag *out);
/* With tracking on, the fused push also sums |v|^2 and v per species, so a
 * per-step ohpic_diagnostics reads them instead of making a second pass over
 * the particles. */
int ohpic_set_energy_tracking(ohpic_ctx *ctx, int enable);

/* Fault injection for tests of the bounded device wait (no reference
 * counterpart).  A push stages each tile's E box into shared memory with one
 * TMA copy and waits for it at most `polls` polls of its mbarrier (default
 * 2^22).  With polls = 0 every wait gives up at once: the kernel gathers from
 * global memory instead, so the particles come out the same, waits the copy out
 * before the CTA finishes, and the next call that synchronises (download,
 * diagnostics, ohpic_synchronize) returns OHPIC_ERR_TIMEOUT. */
int ohpic_set_tma_wait_limit(ohpic_ctx *ctx, uint32_t polls);

/* The per-particle bindings of the reference cannot be served from device
 * memory; the batched calls above replace them.  These return
 * OHPIC_ERR_UNSUPPORTED so a caller that still loops per particle fails loudly. */
int ohpic_move_one(ohpic_ctx *ctx, double *particle, double qm, const double *eb, double dt);
int ohpic_scatter_one(ohpic_ctx *ctx, const double *particle, double amount, int ps);

/* Copies the last error message (NUL-terminated, truncated to len). */
int ohpic_last_error(const ohpic_ctx *ctx, char *buf, size_t len);
/* Message of a status code. */
const char *ohpic_status_string(int status);

int ohpic_synchronize(ohpic_ctx *ctx);
/* The context's cudaStream_t, for callers that order their own work after it. */
int ohpic_get_stream(ohpic_ctx *ctx, void **stream);

/* Launch-shape tuning (no reference counterpart: the reference has no device
 * kernels).  The autotuner (ohhelppic3d_gb300.autotune) times candidate values
 * on the run's own particles and keeps the fastest per grid size. */
enum {
    OHPIC_DEPOSIT_RUNS = 0,       /* warp segmented reduction over runs of equal cells (shuffles) */
    OHPIC_DEPOSIT_UNIFORM = 1,    /* whole-warp hardware reduce when all lanes share a cell, else runs */
    OHPIC_DEPOSIT_MATCH = 2,      /* match lanes by cell, hardware reduce per group */
    OHPIC_DEPOSIT_GROUPS = 3,     /* one whole-warp hardware reduce per distinct cell (up to 3), then runs */
    OHPIC_DEPOSIT_LANES = 4       /* no warp combining: each lane adds its register sums to the shared box
                                     (the default; with four particles per lane the same-address shared
                                     atomics cost less than the shuffles) */
};
typedef struct ohpic_tuning {
    int32_t tile[3];            /* cells per tile edge; powers of two dividing n, <= 64 */
    int32_t halo;               /* cells staged around a tile, 0..4 */
    int32_t split;              /* CTAs per (species, tile), 1..64 */
    int32_t deposit;            /* OHPIC_DEPOSIT_* (FP32 form) */
    int32_t sort_every;         /* cell sort cadence in steps; 0 = only explicit sorts */
    int32_t lane_particles;     /* FP32 push: consecutive particles per lane, 2 or 4 */
    int32_t sort_lead;          /* FP32 form, 0..4096: the cell sort files each particle under
                                   the cell it reaches after this many steps of straight-line
                                   motion (0: its current cell), so that a sort cycle's
                                   particles stay closer to their tile's staged box */
} ohpic_tuning;
int ohpic_get_tuning(ohpic_ctx *ctx, ohpic_tuning *out);
/* Changing tile or halo re-lays out the staged E field: the next push solves
 * again and the next step sorts again. */
int ohpic_set_tuning(ohpic_ctx *ctx, const ohpic_tuning *tuning);

/* Instrumentation: kernel launches issued by this context so far, and the
 * summed CUDA-event duration of the fused push kernel (enable first). */
int ohpic_set_push_timing(ohpic_ctx *ctx, int enable);
int ohpic_stats(ohpic_ctx *ctx, int64_t *launches, int64_t *push_launches, double *push_ms);
/* Device bytes held by the context. */
int ohpic_memory(ohpic_ctx *ctx, int64_t *device_bytes);

/* Field solve on a bounded block with a boundary kind per axis: the reference's
 * t_PoissonFieldSolver with non-periodic kinds for one rank
 * (src/field_solver/poisson_field_solver.f90:34-175 over
 * src/field_solver/poisson/poisson_solver3d.f90:28-207 and the FFTW r2r kinds,
 * logical ranges and normalisers of src/field_solver/fft/fftw3/mpi_fftw3_solver.f90:151-236).
 * The block is the reference's global block: nodes 0..n[d] on every axis,
 * (n[0]+1)(n[1]+1)(n[2]+1) doubles with x fastest.  Kinds follow
 * src/field_solver/field_boundary_type.f90:21-71; boundary_values is the
 * reference's boundary_values(2,3) (lo_x, hi_x, lo_y, hi_y, lo_z, hi_z; null = 0).
 *
 * OHPIC_TABLE_AS_WRITTEN reproduces the reference: it divides by the sum of the
 * squared per-axis wave numbers indexed by global node (poisson_solver3d.f90:62-78,
 * whose Dirichlet and Neumann entries are eigenvalues 2(cos t - 1), so their
 * squares are not Laplacian eigenvalues), adds the wall terms of :81-102 to the
 * block's first and last node planes (a Dirichlet wall's plane is outside the
 * transform, so its value has no effect), and zeroes element (0,0,0) of the
 * block when every logical range starts at node 0.  OHPIC_TABLE_CORRECTED divides
 * by the discrete Laplacian's own eigenvalues (sum_d 2 - 2 cos theta_d; periodic
 * axes as written), zeroes only a null mode, takes a Dirichlet value as the wall
 * potential (entering the adjacent interior node) and a Neumann value as the
 * reference's pure-Neumann term (2 bv low, -2 bv high).  Both solve
 * -laplacian(phi) = rho with dx = 1 and use the reference's pi literal.
 * Outside the transformed range, phi holds a periodic axis' image of node 0 at
 * node n and a Dirichlet wall's potential (0 as written).  e (nullable) receives
 * three such blocks, E = -grad phi by the reference's central difference (one-sided
 * at the walls of non-periodic axes).  Grids: n[d] >= 1 (>= 2 for Dirichlet),
 * at most 4096. */
enum { OHPIC_BC_PERIODIC = 0, OHPIC_BC_DIRICHLET = 1, OHPIC_BC_NEUMANN = 2, OHPIC_BC_DIRICHLET_NEUMANN = 3,
       OHPIC_BC_NEUMANN_DIRICHLET = 4 };
enum { OHPIC_TABLE_AS_WRITTEN = 0, OHPIC_TABLE_CORRECTED = 1 };
typedef struct ohpic_poisson ohpic_poisson;
/* Replaces new_PoissonFieldSolver (poisson_field_solver.f90:34-88). */
int ohpic_poisson_create(const int32_t n[3], const int32_t kinds[3], const double boundary_values[6],
                         int32_t table, int32_t device, ohpic_poisson **out);
int ohpic_poisson_destroy(ohpic_poisson *solver);
/* t_FieldSolver%solve (poisson_field_solver.f90:90-175) on host arrays; synchronous. */
int ohpic_poisson_solve(ohpic_poisson *solver, const double *rho, double *phi, double *e);
/* The same on device arrays, ordered on `stream` (a cudaStream_t; 0 is the
 * default stream, as everywhere in CUDA); returns without synchronising. */
int ohpic_poisson_solve_device(ohpic_poisson *solver, const double *rho, double *phi, double *e, void *stream);
int ohpic_poisson_last_error(const ohpic_poisson *solver, char *buf, size_t len);

/* CIC deposit that allocates no device memory (no counterpart in the reference).
 * For callers that cannot let a library allocate GPU memory, e.g. codes that size
 * all device memory once through their own pool and treat a later cudaMalloc as an
 * error.  x, y, z (n device doubles, positions in cells, wrapped periodically into
 * [0, n); non-finite positions deposit nothing) and rho (nx*ny*nz device doubles,
 * x fastest) are the caller's; the call adds charge * CIC(x, y, z) to rho on
 * `stream` (a cudaStream_t, 0 = default) and returns without synchronising.
 * Weights use the fixed-point deposit of the FP32 form (units of 2^-24 per
 * particle, exact per-particle sum), so the result is independent of atomic order.
 * The only scratch is a static device array of 2^21 nodes (16 MiB), held by every
 * GPU that loads the library until the process exits; larger grids return
 * OHPIC_ERR_CAPACITY.  Every call looks up that array's device address
 * (cudaGetSymbolAddress, which allocates nothing) in the current device's context,
 * so a device reset between calls is harmless.  Every call on a device
 * shares the array and leaves it cleared, so calls that overlap on the GPU (two
 * streams, or two host threads) race and corrupt each other's results. */
int ohpic_scatter_noalloc(const double *x, const double *y, const double *z, int64_t n, double charge,
                          int32_t nx, int32_t ny, int32_t nz, int32_t weights, double *rho, void *stream);

#ifdef __cplusplus
}
#endif
#endif
