/*
 * ohpic_subdomain.h -- one MPI rank's OhHelp subdomain of the particle path,
 * resident on that rank's GPU (plain FP64 form).
 *
 * In the reference every rank owns a block of a periodic global grid (its
 * primary subdomain, src/ohhelp/ohhelp.f90:90-126, ranges in
 * subdomain_range(:, :, ps) of src/ohhelp/ohfield.f90:53-72) and one mainstep is
 * (src/ohhelppic3d.f90:286-381):
 *
 *   scatter of the block's particles into rho      :311-320  (to_local_position, ohfield.f90:199-206)
 *   field solve over all ranks                     :323      (MPI FFTW, border exchanges of OhHelp)
 *   interp + Boris + correct_particle + boundaries :334-358  (ohhelp.f90:414-428 gives each particle
 *                                                             the neighbour that now owns it)
 *   correct_load_balancing / transbound            :366-374  (ohhelp.f90:299-337 moves the particles
 *                                                             to their new owners)
 *
 * This header gives a rank the device half of that loop: its particles stay in
 * device memory, the deposit and the move run on the GPU, and only what OhHelp
 * exchanges crosses to the host -- the block's rho (with the upper ghost plane
 * the neighbours reduce), the block's E (with the node the gather needs past the
 * upper face), and the particles that left the block.  OhHelp, MPI and the
 * global field solve stay on the host, as they do in the reference.
 *
 * Conventions are those of ohpic.h: int status (OHPIC_OK or OHPIC_ERR_*),
 * host arrays borrowed for the call, work ordered on the subdomain's own stream,
 * one subdomain per host thread.  Positions are global (cells, dx = 1).
 */
#ifndef OHPIC_SUBDOMAIN_H
#define OHPIC_SUBDOMAIN_H

#include <stddef.h>
#include <stdint.h>

#include "ohpic.h"

#ifdef __cplusplus
extern "C" {
#endif

/* One particle record as OhHelp moves it between ranks: the reference's
 * oh_particle (x, y, z, vx, vy, vz, pid, nid, spec; used at
 * particle_mover_boris.f90:45,54-62 and particle_injector_with_distribution.f90:196-201).
 * spec is the species number 1..nspecies as in the reference.  nid is filled by
 * ohpic_sub_take_emigrants with the direction the particle left the block in:
 * (dx+1) + 3(dy+1) + 9(dz+1), d in {-1, 0, +1} per axis (13 = stayed). */
typedef struct ohpic_particle {
    double x, y, z, vx, vy, vz;
    int64_t pid;
    int32_t nid;
    int32_t spec;
} ohpic_particle;

typedef struct ohpic_subdomain ohpic_subdomain;

/* A rank's block: cells lo[d] .. lo[d] + m[d] - 1 of the periodic grid
 * cfg->nx, ny, nz (1 <= m[d], lo[d] + m[d] <= n[d]).  From cfg it takes the
 * grid, species, qm, q, b0, weights, capacity (per species, for this block) and
 * device; precision must be OHPIC_FP64.  Replaces the rank-local part of
 * new_OhHelp / ohhelp_initialize (ohhelp.f90:90-242). */
int ohpic_sub_create(const ohpic_config *cfg, const int32_t lo[3], const int32_t m[3], ohpic_subdomain **out);
int ohpic_sub_destroy(ohpic_subdomain *sd);

/* Appends n records (initial load, or the arrivals of a transbound) to their
 * species.  A record outside the block, or with a non-finite coordinate, fails
 * with OHPIC_ERR_BOUNDS / OHPIC_ERR_NONFINITE and nothing is appended. */
int ohpic_sub_append(ohpic_subdomain *sd, const ohpic_particle *p, int64_t n);
int ohpic_sub_count(ohpic_subdomain *sd, int species, int64_t *n);
/* The species' particles (spec 1-based, nid 13). */
int ohpic_sub_download(ohpic_subdomain *sd, int species, ohpic_particle *out, int64_t capacity, int64_t *n_out);

/* t_Scatter%scatter over the block's particles (linear_scatter.f90:22-55 after
 * to_local_position): rho receives the block's nodes lo .. lo + m inclusive,
 * (m[0]+1)(m[1]+1)(m[2]+1) doubles with x fastest.  The planes at lo + m are the
 * ghost contributions that belong to the upper neighbours (OhHelp's
 * oh3_reduce_field / exchange_borders add them, ohhelp.f90:355-369).  The
 * deposit is the 2^-48 fixed-point deposit of the FP64 form, so interior nodes
 * equal a single-domain ohpic_scatter bit for bit.  Synchronises. */
int ohpic_sub_scatter(ohpic_subdomain *sd, double *rho);

/* The block's E for the next move: three blocks of (m[0]+1)(m[1]+1)(m[2]+1)
 * doubles (Ex, Ey, Ez) over nodes lo .. lo + m, x fastest -- the part of the
 * reference's eb(1:3, -1:m+2, ...) the CIC gather reads (ohfield_factory.f90:130). */
int ohpic_sub_set_e(ohpic_subdomain *sd, const double *e);

/* t_Interpolator%interp + t_ParticleMover%move (Boris) + t_ParticleBoundaries%apply
 * twice over the block's particles, in the reference's operation order (the
 * strict FP64 arithmetic of ohpic_move), then ohhelp_correct_particle: particles
 * whose new position lies outside the block leave the species and wait in the
 * emigrant box.  emigrants (nullable, nspecies values) receives how many left per
 * species.  Synchronises. */
int ohpic_sub_move(ohpic_subdomain *sd, double dt, int64_t *emigrants);

/* The particles the last move took out of the block, every species, with nid
 * set; the host hands them to OhHelp's transbound.  out = NULL with capacity 0
 * only returns the count; a smaller non-zero capacity fails with
 * OHPIC_ERR_CAPACITY.  Either way the records wait until taken, and append,
 * download and the next move refuse to run before. */
int ohpic_sub_take_emigrants(ohpic_subdomain *sd, ohpic_particle *out, int64_t capacity, int64_t *n_out);

int ohpic_sub_last_error(const ohpic_subdomain *sd, char *buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif
