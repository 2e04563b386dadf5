// ohpic_internal.cuh -- shared definitions of the GB300 particle path.
//
// Device data layout (all arrays in HBM, one allocation per array):
//   particles, FP64 form : SoA double x, y, z, vx, vy, vz   (48 B/particle)
//   particles, FP32 form : SoA int32 cell (packed ix | iy<<11 | iz<<22),
//                          float ox, oy, oz in [0,1), float vx, vy, vz (28 B/particle)
//   ids                  : uint32 per particle, moved only by the sort
//   species s occupies [seg[s], seg[s] + cap[s]) of every particle array; segment
//   starts are multiples of kSegAlign so vector loads stay aligned.
//   rho, phi             : nx*ny*nz reals, x fastest
//   E                    : node-padded AoS, 4 reals per node (Ex, Ey, Ez, 0) over nodes
//                          -halo..n+halo on every axis (periodic ghosts), so a tile
//                          plus its halo is one dense box (staged by TMA)
//   spectrum             : nz*ny*(nx/2+1) complex (cuFFT R2C layout); green: same, FP64
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/ohpic.h"

namespace ohpic {

constexpr int kSegAlign = 64;       // particles; keeps every species segment 256-B aligned
constexpr int kMaxHalo = 4;
// FP32 push with four particles per lane: per-thread prefetch stage in shared memory
// (7 arrays x 256 threads x 16 bytes).
constexpr size_t kQuadStageBytes = 7 * 256 * 16;
// Warps per CTA of the tile kernels (256 threads).
constexpr int kTileWarps = 8;
// FP32-form deposit: CIC weights in units of 2^-24 (the 8 weights of a particle sum to exactly 2^24).
constexpr float kWeightScale = 16777216.0f;
constexpr double kWeightUnit = 1.0 / 16777216.0;

// Packed FP32-form cell index: 11 bits x, 11 bits y, 10 bits z.
constexpr int kCellBitsX = 11, kCellBitsY = 11, kCellBitsZ = 10;
constexpr int kMaxNx = 1 << kCellBitsX, kMaxNy = 1 << kCellBitsY, kMaxNz = 1 << kCellBitsZ;

__host__ __device__ inline int32_t pack_cell(int ix, int iy, int iz)
{
    return (int32_t)((uint32_t)ix | ((uint32_t)iy << kCellBitsX) |
                     ((uint32_t)iz << (kCellBitsX + kCellBitsY)));
}
__host__ __device__ inline int cell_x(int32_t c) { return (int)((uint32_t)c & (kMaxNx - 1)); }
__host__ __device__ inline int cell_y(int32_t c) { return (int)(((uint32_t)c >> kCellBitsX) & (kMaxNy - 1)); }
__host__ __device__ inline int cell_z(int32_t c) { return (int)((uint32_t)c >> (kCellBitsX + kCellBitsY)); }

// Grid geometry shared by every kernel (passed by value).
struct Geom {
    int nx, ny, nz;
    int tx, ty, tz;        // tile shape (cells); power-of-two divisors of n
    int ntx, nty, ntz;     // tiles per axis
    int halo;              // cells staged around a tile
    int sx, sy, sz;        // staged nodes per axis: t + 2*halo + 1
    int gx, gy, gz;        // padded E nodes per axis: n + 2*halo + 1
    int64_t ncell;
    int64_t ntile;
    int tile_cells;
    int nxh;               // nx/2 + 1
    int64_t nspec;         // nz*ny*nxh
};

// Per-species constants of the push, all derived on the host in FP64.
struct SpeciesConst {
    double qm, q, dt;
    double dt2;            // dt*0.5 (particle_mover_boris.f90:37)
    double t[3];           // qm*B*dt2 (:42)
    double s[3];           // 2t/(1+|t|^2) (:43)
    double mass;           // q/qm
    double hq;             // qm*dt2 rounded once: the plain FP64 push's half kick is one FMA per component
    // The FP32 push's constants, rounded once on the host from the values
    // above: qm*dt2, dt, t, s.  Read as floats, the kernel never converts (a
    // conversion from double runs on GB300's narrow FP64 pipe).
    float hq32, dt32, t32[3], s32[3];
};

// One FP64 E node (Ex, Ey, Ez, pad), 32-byte aligned.
struct __align__(32) dnode {
    double x, y, z, w;
};

struct PartF64 {
    double *x, *y, *z, *vx, *vy, *vz;
};
struct PartF32 {
    int32_t *cell;
    float *ox, *oy, *oz, *vx, *vy, *vz;
};

// Diagnostics accumulated on the device.
struct DevDiag {
    unsigned long long crossings[3];
    unsigned long long outside;
    double kin[OHPIC_MAX_SPECIES][4];   // sum |v|^2, sum vx, sum vy, sum vz
    double charge;
    double field_energy;
    int err_code;          // first device error (OHPIC_ERR_*), 0 = none
    int err_info;
};

enum PushMode { MODE_PUSH = 0, MODE_MOVE = 1, MODE_DEPOSIT = 2, MODE_INTERP = 3 };

// Arguments of the tiled particle kernels.
struct TileArgs {
    Geom g;
    int nspecies;
    int weights;                       // OHPIC_WEIGHTS_*
    int split;                         // CTAs per (species, tile)
    int deposit;                       // OHPIC_DEPOSIT_* (FP32 form)
    int use_tma;                       // stage the E box with cp.async.bulk.tensor
    int with_energy;                   // accumulate kinetic energy / momentum
    int sorted;                        // tile_begin valid
    int ppl;                           // FP32 push/deposit: particles per lane, 2 or 4
    uint32_t tma_polls;                // bound of the wait for the staged E box (0: give up at once)
    int64_t seg[OHPIC_MAX_SPECIES];
    int64_t count[OHPIC_MAX_SPECIES];
    SpeciesConst sc[OHPIC_MAX_SPECIES];
    const int64_t *tile_begin;         // [nspecies][ntile+1], absolute array indices
    const void *epad;                  // padded E
    void *rho;                         // n^3 (zeroed by the caller for deposit modes); FP64 form
    unsigned long long *wsum;          // [species][n^3] sums of CIC weights, 2^-24 (FP32) or 2^-48 (FP64) fixed point
    double *interp_out;                // MODE_INTERP: 3 per particle slot (absolute index)
    DevDiag *diag;
    int chunk;                         // particles per CTA when unsorted
};

// Sorted 32-byte particle records (sort.cu) read by the push that follows the
// sort, and the ids array that push fills from them (null when ids are not
// tracked).
struct RecIn {
    const int4 *rec;
    uint32_t *ids;
};

// One run of the multi-run push (serve.cu): its tile arguments and current particles.
constexpr int kMaxServeRuns = 512;
struct RunDesc {
    TileArgs a;
    PartF32 p;
};
// Arguments of the multi-run persistent push: runs[r] owns the items
// [item_end[r-1], item_end[r]) of one queue; cursor is zero at launch.  The run
// count is read from device memory, so a captured launch serves any set of runs.
struct MultiPush {
    const RunDesc *runs;
    const int64_t *item_end;
    const int *nruns;
    unsigned long long *cursor;
};

// One (run, species) segment of the multi-run sort (sort.cu, driven by serve.cu).
// Its counters are count[key_base .. key_base + ncell) in one key space shared by
// all segments, so one exclusive scan serves every run.
struct SortSeg {
    Geom g;
    PartF32 p;               // sorted in place, through the record area
    uint32_t *ids;           // may be null
    int4 *rec;               // the run's record area: 32 bytes per particle slot
    int64_t off, count;      // particles [off, off + count) of the run's arrays
    int64_t key_base;
    int64_t *tile_begin;     // ntile + 1 entries, absolute particle indices
    DevDiag *diag;
    float h;                 // sort lead in cells per unit velocity (0: sort by the current cell)
};
constexpr int kMaxSortSegs = kMaxServeRuns * 2;
constexpr int kSortChunk = 8192;   // particles per CTA pass
struct MultiSort {
    const SortSeg *segs;
    const int32_t *chunk_end;   // inclusive prefix of the chunks of every segment
    const int *nseg;            // segment count, in device memory
    uint32_t *count;            // zeroed before the histogram
    uint32_t *start;            // exclusive scan of count
    uint32_t *cursor;           // zeroed before the scatter
};

// Fields of many runs of one grid size (serve.cu): slot k owns the k-th n^3 block
// of rho and phi, the k-th spectrum and padded E, and nsp weight-sum arrays;
// one batched cuFFT plan pair covers every slot.
struct FieldPool {
    Geom g;
    int slots;
    int nsp;                        // weight-sum arrays per slot
    float *rho, *phi;
    cufftComplex *spec;
    float4 *epad;
    unsigned long long *wsum;
    double *green;                  // shared by the slots (same grid)
    double *q;                      // [slot][nsp] species charges
    int *on;                        // [slot] 1 when a run owns the slot
    cufftHandle r2c, c2r;
};

// Host-side context.
}  // namespace ohpic

struct ohpic_ctx {
    ohpic_config cfg;
    ohpic::Geom g;
    int dev;
    cudaStream_t stream;
    int64_t seg[OHPIC_MAX_SPECIES];
    int64_t cap[OHPIC_MAX_SPECIES];
    int64_t count[OHPIC_MAX_SPECIES];
    int64_t total_slots;
    ohpic::SpeciesConst sc[OHPIC_MAX_SPECIES];
    double sc_dt;                       // dt the species constants were built for

    // particle buffers: [cur] holds the particles; the other one is the sort's
    // record area (the sort works in place, so cur stays 0)
    ohpic::PartF64 p64[2];
    ohpic::PartF32 p32[2];
    uint32_t *ids[2];
    // Each particle buffer is one allocation of eight arrays, so it also holds N
    // sort records: FP32 form eight 4-byte arrays (cell, offsets, velocities,
    // ids) = 32-byte records; FP64 form eight 8-byte arrays (positions,
    // velocities, ids, padding) = 64-byte records.
    void *pblock[2];
    int cur;

    // fields
    void *rho, *phi, *epad;
    // The deposit accumulates per-species weight sums in fixed point (2^-24 in
    // the FP32 form, 2^-48 in the FP64 form; integer adds, so the result does not
    // depend on the order of the atomics); the solve turns them into rho.
    unsigned long long *wsum;
    bool rho_from_wsum;
    // TMA description of epad for staging a tile's E box (tma_map.cu).
    CUtensorMap emap;   // carries its own alignment
    bool emap_ok;
    void *emap_for;
    int emap_key[4];
    void *spec;
    double *green;
    cufftHandle plan_r2c, plan_c2r;
    bool plans_made;

    // sort
    uint32_t *cell_count;   // ncell
    uint32_t *cell_stay;    // ncell: the tile-local re-sort's stayer counts
    uint32_t *cell_start;   // ncell + 1
    uint32_t *scan_tmp;
    uint32_t *key_table;    // nx + ny + nz per-axis terms of the tile-major key
    int64_t *tile_begin;    // nspecies * (ntile + 1)
    bool sorted;
    int steps_since_sort;
    // FP32 form: the last sort left every species as cell-sorted 32-byte records
    // in pblock[1 - cur] and the word arrays are stale; the next push reads the
    // records (and writes the arrays), anything else materialises them first.
    bool rec_pending;

    // staging for uploads/downloads
    void *stage;
    int64_t stage_bytes;
    double *interp_buf;
    int64_t interp_cap;

    ohpic::DevDiag *diag;      // device
    ohpic::DevDiag *diag_host; // pinned

    bool rho_valid;
    bool field_valid;
    int64_t steps;
    int split;
    int halo;
    int dep_strategy;           // OHPIC_DEPOSIT_* for the FP32 warp deposit
    int lane_particles;         // FP32 push/deposit: particles per lane (2 or 4)
    int sort_lead;              // FP32 sort: steps of straight-line motion the sort key anticipates
    uint32_t tma_polls;         // polls allowed for the staged E box (ohpic_set_tma_wait_limit)
    bool with_energy;
    bool kin_valid;             // diag->kin holds the sums of the current velocities

    int64_t launches;
    int64_t push_launches;
    bool push_timing;
    std::vector<cudaEvent_t> ev_pool;   // (start, end) pairs around push kernels
    int ev_used;
    double push_ms;
    int64_t device_bytes;
    std::string err;
};

namespace ohpic {

// Host helpers (ohpic_api.cu): geometry of a grid for a tile shape and halo
// (false when it does not fit), and the FP64 Boris constants of one species.
bool make_geom(const ohpic_config &k, const int tile[3], int halo, Geom &g);
void species_consts(const ohpic_config &cfg, int s, double dt, SpeciesConst &k);

// Kernel launchers: dispatch (convert.cu) and the two forms (push_f64.cu, push_f32.cu).
void launch_tiled(ohpic_ctx *c, int mode, int strict);
void launch_tiled_f64(ohpic_ctx *c, const TileArgs &a, int mode, int strict, int64_t blocks, size_t smem);
void launch_tiled_f32(ohpic_ctx *c, const TileArgs &a, int mode, int64_t blocks, size_t smem,
                      const RecIn *rin = nullptr);
// FP32 form: turns the sort's pending records back into the word arrays (no-op
// when none are pending); every entry point that reads or writes particles
// other than the push that consumes the records calls it first.
void materialize_records(ohpic_ctx *c);
cudaError_t launch_multi_f32(cudaStream_t st, int mode, int dep, int ppl, int weights, const MultiPush &m,
                             int grid, size_t smem);
void ensure_emap(ohpic_ctx *c);
// Fields (fields.cu).
int fields_setup(ohpic_ctx *c);
void fields_teardown(ohpic_ctx *c);
int solve_fields(ohpic_ctx *c);
void launch_zero(ohpic_ctx *c, void *p, int64_t bytes);
int pool_green(cudaStream_t st, const Geom &g, double *green);
int pool_solve(cudaStream_t st, const FieldPool &p);
void pool_slot_rho(cudaStream_t st, const FieldPool &p, int slot);
void pool_slot_fields(cudaStream_t st, const FieldPool &p, int slot, double *dst);
void pool_slot_sums(cudaStream_t st, const FieldPool &p, int slot, DevDiag *d);
void launch_field_energy(ohpic_ctx *c);
void field_to_double(ohpic_ctx *c, int which, double *dst);
void field_from_double(ohpic_ctx *c, int which, const double *src);
// Sort (sort.cu).
int sort_particles(ohpic_ctx *c);
int64_t scan_tmp_elems(int64_t n);
// Exclusive scan of n uint32 values; tmp holds scan_tmp_elems(n) values.
int scan_u32(cudaStream_t st, const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp);
// Multi-run sort passes; each returns the number of launches it made.
int launch_sort_hist_multi(cudaStream_t st, const MultiSort &m, int64_t chunks);
int launch_sort_finish_multi(cudaStream_t st, const MultiSort &m, int64_t chunks, int64_t max_ntile,
                             int max_seg, int64_t nkeys, uint32_t *scan_tmp);
// Conversions (convert.cu).
void launch_f64_to_f32(ohpic_ctx *c, const double *stage6, int64_t n, int64_t dst, uint32_t id0,
                       int aos, int64_t stride_doubles);
void launch_f64_soa_from_stage(ohpic_ctx *c, const double *stage, int64_t n, int64_t dst, uint32_t id0,
                               int aos, int64_t stride_doubles);
void launch_to_f64_stage(ohpic_ctx *c, double *stage, int64_t src, int64_t n);
// Six FP64 SoA arrays the kernels read or write directly (device-accessible host
// memory: pinned or registered); a null output array is skipped.
struct Soa6 {
    const double *p[6];
};
struct Soa6w {
    double *p[6];
};
void launch_from_host_soa(ohpic_ctx *c, const Soa6 &s, int64_t n, int64_t dst, uint32_t id0);
void launch_to_host_soa(ohpic_ctx *c, const Soa6w &out, int64_t src, int64_t n);
// The device address of a host array the GPU can reach (pinned or registered), else null.
const void *device_view(const void *host);
void launch_kinetic(ohpic_ctx *c);
// Device-side initial conditions (init.cu).
int init_particles(ohpic_ctx *c, uint64_t initstate, uint64_t initseq, uint64_t advance,
                   const ohpic_species_init *spi, int64_t *counts);
// The injector over explicit buffers: species s goes to [seg[s], seg[s] + count)
// of p64/p32 (by precision).  counts_only draws the random_fix counts on the host
// and launches nothing.
struct DrawSpec {
    cudaStream_t stream = nullptr;
    int precision = OHPIC_FP32;
    int n[3] = {0, 0, 0};
    uint64_t initstate = 0, initseq = 0, advance = 0;
    int nspecies = 0;
    const ohpic_species_init *spi = nullptr;
    const int64_t *seg = nullptr;
    const int64_t *cap = nullptr;
    PartF64 p64{};
    PartF32 p32{};
    uint32_t *ids = nullptr;
    bool counts_only = false;
    int64_t *launches = nullptr;
};
int draw_particles(const DrawSpec &d, int64_t *counts, std::string *err);

}  // namespace ohpic

#define OHPIC_CUDA_TRY(c, expr)                                                         \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            (c)->err = std::string(#expr) + ": " + cudaGetErrorString(e_);              \
            return OHPIC_ERR_CUDA;                                                      \
        }                                                                               \
    } while (0)
