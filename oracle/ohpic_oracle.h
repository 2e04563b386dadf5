/*
 * ohpic_oracle.h -- CPU restatement of ohhelppic3d's per-timestep particle path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness checker for the
 * GPU library (ohhelppic3d_gb300) and the timed CPU baseline.  Only the test
 * suite, the smoke check and the benchmark's CPU-baseline leg load it; the
 * product path never does.
 *
 * It restates, in plain C (FP64, no FMA contraction), the reference's
 * Fortran path:
 *   deposit   src/scatter/linear_scatter.f90:32-53 (driven by src/ohhelppic3d.f90:311-320)
 *   solve     src/field_solver/poisson/poisson_solver3d.f90:62-78,104-117,147,184-205
 *             src/field_solver/fft/fftw3/mpi_fftw3_solver.f90:166-173,235
 *   E stencil src/field_solver/poisson_field_solver.f90:131-171
 *   gather    src/interpolator/linear_interpolator.f90:33-67
 *   push      src/particle_mover/particle_mover_boris.f90:37-62
 *   wrap      src/particle_boundary/periodic_particle_boundary.f90:42-53 (applied twice,
 *             src/ohhelppic3d.f90:353,355)
 *   init      src/ohhelppic3d.f90:111-112, particle_injector_with_distribution.f90:51-69,
 *             position_random_uniform_distribution.f90:38-41,
 *             velocity_maxwell_distribution3d.f90:41-56, random_generator.f90:45-58
 *   RNG       lib/pcg-c (pcg32 = setseq_64 / xsh_rr_64_32; pcg32_double.c:60-63),
 *             restated from the published PCG algorithm.
 *
 * Documented deviations shared with the GPU library:
 *   D1 CIC weights: the reference gives node i the weight r = x - floor(x) and
 *      node i+1 the weight 1-r (linear_interpolator.f90:54-64, linear_scatter.f90:41-52).
 *      ORC_WEIGHTS_REFERENCE keeps that; ORC_WEIGHTS_STANDARD swaps it to textbook CIC.
 *   D2 E stencil reads phi component 1 for all three axes (the reference indexes
 *      phi%values(2..3,...) of a one-element field, poisson_field_solver.f90:141-144).
 *   D3 Maxwellian standard deviation is vth (the reference multiplies by 2,
 *      velocity_maxwell_distribution3d.f90:52-54); an optional drift is added after the clip.
 *   D4 B is a uniform constant B0 passed to Boris (the reference never fills eb(4:6)).
 *   D5 the periodic ghost node n of rho is folded into node 0 after every deposit.
 *   D7 particles per species = ppc * (cells covered by the species' position range).
 */
#ifndef OHPIC_ORACLE_H
#define OHPIC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_SPECIES 8

enum { ORC_WEIGHTS_REFERENCE = 0, ORC_WEIGHTS_STANDARD = 1 };
enum { ORC_RHO = 0, ORC_PHI = 1, ORC_EX = 2, ORC_EY = 3, ORC_EZ = 4 };

/* PCG32 (64-bit state, selectable stream, XSH-RR output). */
typedef struct {
    uint64_t state;
    uint64_t inc;
} orc_pcg32;

void orc_pcg32_srandom(orc_pcg32 *rng, uint64_t initstate, uint64_t initseq);
uint32_t orc_pcg32_random(orc_pcg32 *rng);
void orc_pcg32_advance(orc_pcg32 *rng, uint64_t delta);
double orc_pcg32_double(orc_pcg32 *rng);
/* Fills out[0..n) with consecutive draws (KAT helper). */
void orc_pcg32_fill(uint64_t initstate, uint64_t initseq, uint64_t advance,
                    uint32_t *out, int64_t n);

typedef struct {
    int32_t nx, ny, nz;
    int32_t nspecies;
    int32_t weights;          /* ORC_WEIGHTS_* */
    int32_t pad0;
    double dt;
    double b0[3];             /* uniform magnetic field (D4) */
    double qm[ORC_MAX_SPECIES];     /* charge-to-mass ratio per species */
    double q[ORC_MAX_SPECIES];      /* charge per macro-particle per species */
    int64_t capacity[ORC_MAX_SPECIES];
} orc_config;

/* Injector parameters for one species (reference injector + D3/D7). */
typedef struct {
    double ppc;               /* macro-particles per cell inside the range */
    double vth;               /* Maxwellian standard deviation (D3) */
    double drift[3];          /* added after the +-6 vth clip */
    double lo[3], hi[3];      /* position range; clipped to [0, n] */
} orc_species_init;

typedef struct {
    int64_t count[ORC_MAX_SPECIES];
    int64_t crossings[3];     /* particles that wrapped along x, y, z in the last push */
    double total_charge;      /* sum of rho over nodes */
    double field_energy;      /* 0.5 * sum |E|^2 over nodes */
    double kinetic_energy;    /* sum 0.5 * (q/qm) * |v|^2 */
    double momentum[3];       /* sum (q/qm) * v */
} orc_diag;

typedef struct orc_sim orc_sim;

orc_sim *orc_create(const orc_config *cfg);
void orc_destroy(orc_sim *s);
/* Number of OpenMP threads the oracle uses (1 = the sequential reference order). */
void orc_set_threads(orc_sim *s, int nthreads);
int orc_max_threads(void);

/* Injector: seeds (initstate, initseq), then advance(rank_advance), then per species
 * one random_fix draw followed by 3 position and 4 velocity draws per particle. */
int orc_init_particles(orc_sim *s, uint64_t initstate, uint64_t initseq,
                       uint64_t rank_advance, const orc_species_init *sp);

int orc_set_particles(orc_sim *s, int species, const double *x, const double *y,
                      const double *z, const double *vx, const double *vy,
                      const double *vz, int64_t n);
int64_t orc_get_particles(const orc_sim *s, int species, double *x, double *y,
                          double *z, double *vx, double *vy, double *vz);
int64_t orc_count(const orc_sim *s, int species);

/* Fields are nx*ny*nz doubles, x fastest. */
void orc_get_field(const orc_sim *s, int which, double *out);
void orc_set_field(orc_sim *s, int which, const double *in);

void orc_deposit(orc_sim *s);              /* rho from current particles */
void orc_solve(orc_sim *s);                /* phi and E from rho */
void orc_push(orc_sim *s);                 /* gather + Boris + position + wrap x2 */
/* nsteps x (deposit, solve, push), the reference mainstep order. */
void orc_step(orc_sim *s, int nsteps);
void orc_diagnostics(orc_sim *s, orc_diag *d);

/* Building blocks, exposed for known-answer tests. */
void orc_interp_one(const orc_sim *s, double x, double y, double z, double e[3]);
void orc_boris_one(double qm, const double e[3], const double b[3], double dt,
                   double pos[3], double vel[3]);
void orc_wrap(int n, double *p);
/* In-place 3-D complex DFT (sign -1 forward, +1 backward, unnormalised) of an
 * nx*ny*nz interleaved (re, im) array, x fastest. */
void orc_fft3d(double *data, int nx, int ny, int nz, int sign);
/* Green factor 1/sum_d (2 sin(pi k_d / n_d))^2 with the reference's pi literal
 * (poisson_solver3d.f90:104-117); returns 0 for k = 0. */
double orc_green(int kx, int ky, int kz, int nx, int ny, int nz);

/* Field solve on a bounded block with per-axis boundary kinds: the reference's
 * poissonSolver3d_solve (src/field_solver/poisson/poisson_solver3d.f90:134-207)
 * over the FFTW r2r transforms of src/field_solver/fft/fftw3/mpi_fftw3_solver.f90
 * (kinds, logical ranges and normalisers :151-207, backward normalisation :235),
 * the wave-number table of poisson_solver3d.f90:56-78,104-132 and the wall terms
 * of :81-102, for one rank whose block is the global block 0..n per axis.
 *
 * Kinds (src/field_solver/field_boundary_type.f90:21-71): */
enum { ORC_BC_PERIODIC = 0, ORC_BC_DIRICHLET = 1, ORC_BC_NEUMANN = 2, ORC_BC_DIRICHLET_NEUMANN = 3,
       ORC_BC_NEUMANN_DIRICHLET = 4 };
/* rho, phi: (n[0]+1)(n[1]+1)(n[2]+1) doubles, x fastest, nodes 0..n per axis.
 * bv: boundary_values(2,3) in Fortran order (lo_x, hi_x, lo_y, hi_y, lo_z, hi_z).
 * corrected = 0 follows the reference as written: the table is the sum of the
 * squared per-axis wave numbers indexed by global node, the wall terms go to the
 * block's first and last node planes, and element (0,0,0) of the block is zeroed
 * when every logical range starts at node 0.  corrected = 1 divides by the
 * Laplacian's own eigenvalues at the logical index (sum_d 2 - 2 cos(theta_d); the
 * periodic axes keep (2 sin(pi k/n))^2), zeroes only a null mode, takes a
 * Dirichlet wall value as the wall's potential (its term goes to the adjacent
 * interior node), a Neumann value as in the reference's pure-Neumann terms (2 bv
 * at a low wall, -2 bv at a high one) on either mixed kind, and no term on a
 * periodic axis.  phi at nodes outside the transformed range: a periodic axis'
 * node n is the image of node 0; a Dirichlet wall holds 0 (as written) or its
 * value (corrected).  e (nullable): 3 blocks of the same size, E = -grad phi by
 * the reference's central difference 0.5*((phi[i-1] - phi[i]) + (phi[i] -
 * phi[i+1])), wrapped on periodic axes, one-sided (phi[0] - phi[1], phi[n-1] -
 * phi[n]) at the walls of the others.  Returns 0, or -1 for bad arguments. */
int orc_poisson_bc(const int n[3], const int kinds[3], const double bv[6], int corrected, const double *rho,
                   double *phi, double *e);
/* One-dimensional unnormalised real transform by its defining sum, FFTW's
 * conventions: kind 0 R2HC, 1 HC2R, 2 RODFT00, 3 REDFT00, 4 RODFT01, 5 RODFT10,
 * 6 REDFT01, 7 REDFT10. */
void orc_r2r_1d(int kind, const double *x, double *y, int n);

#ifdef __cplusplus
}
#endif
#endif
