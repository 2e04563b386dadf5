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
    int64_t seg[OHPIC_MAX_SPECIES];
    int64_t count[OHPIC_MAX_SPECIES];
    SpeciesConst sc[OHPIC_MAX_SPECIES];
    const int64_t *tile_begin;         // [nspecies][ntile+1], absolute array indices
    const void *epad;                  // padded E
    void *rho;                         // n^3 (zeroed by the caller for deposit modes); FP64 form
    unsigned long long *wsum;          // FP32 form: [species][n^3] sums of CIC weights, 2^-24 fixed point
    double *interp_out;                // MODE_INTERP: 3 per particle slot (absolute index)
    DevDiag *diag;
    int chunk;                         // particles per CTA when unsorted
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

    // particle buffers: [0] current, [1] sort target
    ohpic::PartF64 p64[2];
    ohpic::PartF32 p32[2];
    uint32_t *ids[2];
    int cur;

    // fields
    void *rho, *phi, *epad;
    // FP32 form: the deposit accumulates per-species weight sums in 2^-24 fixed
    // point (integer adds, so the result does not depend on the order of the
    // atomics); the solve turns them into rho.
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
    uint32_t *cell_start;   // ncell + 1
    uint32_t *scan_tmp;
    int64_t *tile_begin;    // nspecies * (ntile + 1)
    bool sorted;
    int steps_since_sort;

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

// Kernel launchers: dispatch (convert.cu) and the two forms (push_f64.cu, push_f32.cu).
void launch_tiled(ohpic_ctx *c, int mode, int strict);
void launch_tiled_f64(ohpic_ctx *c, const TileArgs &a, int mode, int strict, int64_t blocks, size_t smem);
void launch_tiled_f32(ohpic_ctx *c, const TileArgs &a, int mode, int64_t blocks, size_t smem);
void ensure_emap(ohpic_ctx *c);
// Fields (fields.cu).
int fields_setup(ohpic_ctx *c);
void fields_teardown(ohpic_ctx *c);
int solve_fields(ohpic_ctx *c);
void launch_zero(ohpic_ctx *c, void *p, int64_t bytes);
void launch_field_energy(ohpic_ctx *c);
void field_to_double(ohpic_ctx *c, int which, double *dst);
void field_from_double(ohpic_ctx *c, int which, const double *src);
// Sort (sort.cu).
int sort_particles(ohpic_ctx *c);
int64_t scan_tmp_elems(int64_t n);
// Conversions (convert.cu).
void launch_f64_to_f32(ohpic_ctx *c, const double *stage6, int64_t n, int64_t dst, uint32_t id0,
                       int aos, int64_t stride_doubles);
void launch_f64_soa_from_stage(ohpic_ctx *c, const double *stage, int64_t n, int64_t dst, uint32_t id0,
                               int aos, int64_t stride_doubles);
void launch_to_f64_stage(ohpic_ctx *c, double *stage, int64_t src, int64_t n);
void launch_kinetic(ohpic_ctx *c);
// Device-side initial conditions (init.cu).
int init_particles(ohpic_ctx *c, uint64_t initstate, uint64_t initseq, uint64_t advance,
                   const ohpic_species_init *spi, int64_t *counts);

}  // namespace ohpic

#define OHPIC_CUDA_TRY(c, expr)                                                         \
    do {                                                                                \
        cudaError_t e_ = (expr);                                                        \
        if (e_ != cudaSuccess) {                                                        \
            (c)->err = std::string(#expr) + ": " + cudaGetErrorString(e_);              \
            return OHPIC_ERR_CUDA;                                                      \
        }                                                                               \
    } while (0)
