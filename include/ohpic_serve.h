/* ohpic_serve.h -- continuous-batching server for many small periodic runs.
 *
 * No reference counterpart: the reference runs one simulation per MPI job
 * (src/ohhelppic3d.f90:311-358).  The server accepts independent runs while
 * others are on the GPU.  Each run is admitted by its HBM footprint, and every
 * admitted run is advanced one step per tick:
 *   - the fields of all runs of one grid size are solved together: batched
 *     cuFFT plus pooled kernels over the size class's field slots;
 *   - the particles of all runs are pushed by one persistent kernel that pulls
 *     (run, species, tile) items from a shared queue;
 *   - the cell sort of all runs is one histogram, one scan and one scatter.
 * A tick is captured once into a CUDA graph and replayed until the set of
 * runs changes.
 *
 * Runs use the FP32 precision form (ohpic.h, OHPIC_FP32) with the same device
 * injector as ohpic_init_particles.  A run's result does not depend on which
 * other runs share the GPU:
 *   - the deposit is integer fixed point;
 *   - every particle is advanced independently;
 *   - a slot's transform is the same batched plan whatever the other slots hold.
 *
 * Threading: one worker thread per server drives the GPU.  submit, poll,
 * result, wait and stats may be called from any host thread.
 */
#ifndef OHPIC_SERVE_H
#define OHPIC_SERVE_H

#include <stddef.h>
#include <stdint.h>

#include "ohpic.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ohpic_server ohpic_server;

typedef struct {
    int32_t device;
    int32_t max_active;          /* runs on the GPU at once (<= 512; 0 = 512) */
    int64_t hbm_budget;          /* bytes for run state and field pools (0 = 60% of free memory) */
    int32_t slots_per_pool;      /* field slots per grid-size pool (0 = 16) */
    int32_t sort_every;          /* ticks between cell sorts of all runs (0 = 8) */
    int32_t use_graphs;          /* 1: replay each tick as a captured CUDA graph */
    int32_t weights;             /* OHPIC_WEIGHTS_* for every run */
    int32_t tile;                /* largest tile edge in y and z (0 = 8); per grid, the largest power of
                                    two <= tile dividing the edge */
    int32_t halo;                /* staged halo cells (0 = 1) */
    int32_t deposit;             /* OHPIC_DEPOSIT_* */
    int32_t max_species;         /* species per run the pools hold (0 = 2, <= OHPIC_MAX_SPECIES) */
    int32_t lane_particles;      /* consecutive particles per lane in the push, 2 or 4 (0 = 4) */
    int32_t tile_x;              /* largest tile edge along x (0 = 2 x tile, at most 64): a tile twice as
                                    long in x halves the halo share of the staged box and still
                                    leaves two CTAs per SM */
    int32_t sort_lead;           /* 0..4096: the cell sort files each particle under the cell it reaches
                                    after this many steps of straight-line motion (0: its current cell;
                                    the default config: half the default sort cadence) */
    int32_t reserved[3];
} ohpic_serve_config;

typedef struct {
    int32_t nx, ny, nz, nspecies;
    double dt;
    double b0[3];
    double qm[OHPIC_MAX_SPECIES];
    double q[OHPIC_MAX_SPECIES];
    ohpic_species_init species[OHPIC_MAX_SPECIES];
    uint64_t seed_state, seed_seq;   /* pcg32 stream of the injector, e.g. (42, 52 + i) */
    int64_t nsteps;
    int32_t keep_fields;              /* keep rho, phi, Ex, Ey, Ez (FP64) of the final state */
    int32_t keep_particles;           /* keep x, y, z, vx, vy, vz (FP64) in injection order */
} ohpic_run_request;

typedef struct {
    int64_t id;
    int32_t status;                  /* OHPIC_OK or the run's error */
    int32_t done;                    /* 1 once the result is final */
    int64_t steps;                   /* steps advanced */
    int64_t particles;
    double submit_s, admit_s, finish_s;   /* server clock, seconds since ohpic_serve_create */
    ohpic_diag diag;                 /* counts, crossings over the run, charge, field and kinetic energy */
} ohpic_run_result;

typedef struct {
    int64_t submitted, admitted, completed, failed;
    int64_t active, pending;
    int64_t ticks, sort_ticks;
    int64_t particle_steps;
    int64_t graph_captures, graph_launches;
    int64_t launches;                /* kernels launched (graph replays count their kernels) */
    int64_t bytes_in_use, bytes_peak, budget;
    int32_t pools;
    int32_t reserved;
} ohpic_serve_stats;

void ohpic_serve_config_default(ohpic_serve_config *cfg);
void ohpic_run_request_default(ohpic_run_request *req);
int ohpic_serve_create(const ohpic_serve_config *cfg, ohpic_server **out);
/* Stops the worker after the runs already on the GPU; pending runs are dropped. */
int ohpic_serve_destroy(ohpic_server *s);
/* Queues a run.  OHPIC_ERR_INVALID for a bad request; OHPIC_ERR_CAPACITY if the
 * run alone exceeds the budget. */
int ohpic_serve_submit(ohpic_server *s, const ohpic_run_request *req, int64_t *id);
/* Ids of runs completed since the last poll (at most cap); *n = how many. */
int ohpic_serve_poll(ohpic_server *s, int64_t *ids, int32_t cap, int32_t *n);
/* Blocks until every submitted run has completed or timeout_s passed
 * (OHPIC_ERR_TIMEOUT).  timeout_s <= 0 waits without limit. */
int ohpic_serve_wait(ohpic_server *s, double timeout_s);
/* The result of run id.  fields: 5*nx*ny*nz doubles (rho, phi, Ex, Ey, Ez) when the
 * run kept them, else ignored; particles: per species 6*count doubles (x, y, z,
 * vx, vy, vz blocks) one species after another, when kept.  Either may be NULL. */
int ohpic_serve_result(ohpic_server *s, int64_t id, ohpic_run_result *res, double *fields, double *particles);
/* Releases a completed run's kept result. */
int ohpic_serve_release(ohpic_server *s, int64_t id);
int ohpic_serve_stats_get(ohpic_server *s, ohpic_serve_stats *st);
int ohpic_serve_last_error(ohpic_server *s, char *buf, size_t len);
/* HBM bytes a run would hold while active (particles, a 32-byte sort record per slot, tile table). */
int64_t ohpic_serve_footprint(const ohpic_serve_config *cfg, const ohpic_run_request *req);

#ifdef __cplusplus
}
#endif

#endif /* OHPIC_SERVE_H */
