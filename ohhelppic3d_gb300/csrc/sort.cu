// sort.cu -- periodic counting sort of every species by tile-major cell index.
//
// No reference counterpart: the reference walks an unsorted oh_particle buffer.
// The sort makes the particles of one tile a contiguous range so the fused push
// can stage that tile's fields in shared memory (push_f32.cu, push_f64.cu).
//
// Per species: histogram of cell keys (global atomics, one per run of adjacent
// lanes with equal keys), exclusive scan of the ncell counters (multi-level
// block scan), tile start table, then a scatter of every particle as one whole
// record (32 bytes in the FP32 form, 64 in the FP64 form) into the second
// buffer's block.  The FP64 form transposes the records back into the first
// buffer's arrays at once; the FP32 form leaves them to the next push, which
// reads the records directly (push_f32.cu), or to materialize_records.  In the
// scatter, lanes of a warp that share a key (grouped with __match_any_sync) take
// consecutive slots in lane order, so a warp's relative order is kept; order
// across warps follows the atomic order.  With a sort lead (FP32 form,
// ohpic_tuning.sort_lead), the key is the cell each particle reaches after that
// many steps of straight-line motion instead of its current cell.
#include <cmath>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;                      // per thread
constexpr int kScanBlock = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t tile_key(const Geom &g, int ix, int iy, int iz)
{
    const int tx = ix / g.tx, ty = iy / g.ty, tz = iz / g.tz;
    const int lx = ix - tx * g.tx, ly = iy - ty * g.ty, lz = iz - tz * g.tz;
    const uint32_t tile = (uint32_t)tx + (uint32_t)g.ntx * ((uint32_t)ty + (uint32_t)g.nty * (uint32_t)tz);
    return tile * (uint32_t)g.tile_cells + (uint32_t)lx + (uint32_t)g.tx * ((uint32_t)ly + (uint32_t)g.ty * lz);
}

// The tile-major key is a sum of one term per axis: with tile (TX, TY, TZ),
//   key = [ (ix/TX) C + ix%TX ] + [ (iy/TY) NTX C + TX (iy%TY) ] + [ (iz/TZ) NTX NTY C + TX TY (iz%TZ) ]
// (C = cells per tile, NTX/NTY tiles per row/plane), so the single-context sort
// looks the three terms up in a table of nx + ny + nz entries built once per
// sort (k_key_table) instead of dividing by the tile shape per particle.
__global__ void k_key_table(Geom g, uint32_t *tab)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t C = (uint32_t)g.tile_cells;
    if (i < g.nx) {
        tab[i] = (uint32_t)(i / g.tx) * C + (uint32_t)(i % g.tx);
    } else if (i < g.nx + g.ny) {
        const int y = i - g.nx;
        tab[i] = (uint32_t)(y / g.ty) * (uint32_t)g.ntx * C + (uint32_t)g.tx * (uint32_t)(y % g.ty);
    } else if (i < g.nx + g.ny + g.nz) {
        const int z = i - g.nx - g.ny;
        tab[i] = (uint32_t)(z / g.tz) * (uint32_t)g.ntx * (uint32_t)g.nty * C +
                 (uint32_t)(g.tx * g.ty) * (uint32_t)(z % g.tz);
    }
}

// Key of cell (ix, iy, iz) from the table when there is one, else by division;
// a cell outside the grid flags OHPIC_ERR_BOUNDS and sorts as cell 0.
__device__ __forceinline__ uint32_t cell_key(const Geom &g, const uint32_t *tab, int ix, int iy, int iz, DevDiag *d)
{
    if ((unsigned)ix >= (unsigned)g.nx || (unsigned)iy >= (unsigned)g.ny || (unsigned)iz >= (unsigned)g.nz) {
        if (atomicCAS(&d->err_code, 0, OHPIC_ERR_BOUNDS) == 0) d->err_info = 10;
        ix = iy = iz = 0;
    }
    if (tab) return __ldg(tab + ix) + __ldg(tab + g.nx + iy) + __ldg(tab + g.nx + g.ny + iz);
    return tile_key(g, ix, iy, iz);
}

// FP32 form, sort lead h > 0 (cells per unit velocity): a particle is filed
// under the cell it reaches moving in a straight line for h, cell i + floor(o +
// v h) per axis, wrapped into the grid.  Particles then sit, on average, in
// their tile's box at the middle of a sort cycle instead of at its start, so
// fewer of them leave the staged box by its end.  The histogram and the scatter
// run this same sequence of explicitly rounded operations on the same words,
// so they file every particle under the same key.
__device__ __forceinline__ int lead_axis(int i, float o, float v, float h, int n)
{
    float f = floorf(__fmaf_rn(v, h, o));
    f = fminf(fmaxf(f, -16777216.f), 16777216.f);   // |f| <= 2^24 (a NaN gives -2^24)
    int k = i + (int)f;
    if ((unsigned)k >= (unsigned)n) {
        k %= n;
        if (k < 0) k += n;
    }
    return k;
}

// Cell of a packed FP32 cell c with offsets f[0..2] and velocities f[3..5]
// after the lead h (h == 0: the cell itself); a cell outside the grid flags
// OHPIC_ERR_BOUNDS (site `site`) and sorts as cell 0.
__device__ __forceinline__ void lead_cell(const Geom &g, int32_t c, const float f[6], float h, int site,
                                          DevDiag *d, int &ix, int &iy, int &iz)
{
    ix = cell_x(c), iy = cell_y(c), iz = cell_z(c);
    if ((unsigned)ix >= (unsigned)g.nx || (unsigned)iy >= (unsigned)g.ny || (unsigned)iz >= (unsigned)g.nz) {
        if (atomicCAS(&d->err_code, 0, OHPIC_ERR_BOUNDS) == 0) d->err_info = site;
        ix = iy = iz = 0;
    }
    if (h != 0.f) {
        ix = lead_axis(ix, f[0], f[3], h, g.nx);
        iy = lead_axis(iy, f[1], f[4], h, g.ny);
        iz = lead_axis(iz, f[2], f[5], h, g.nz);
    }
}

template <bool F32>
__device__ __forceinline__ uint32_t particle_key(const Geom &g, const uint32_t *tab, const PartF64 &p64,
                                                 const PartF32 &p32, int64_t i, float h, DevDiag *d)
{
    if (F32) {
        const int32_t c = p32.cell[i];
        if (h == 0.f) return cell_key(g, tab, cell_x(c), cell_y(c), cell_z(c), d);
        const float f[6] = {p32.ox[i], p32.oy[i], p32.oz[i], p32.vx[i], p32.vy[i], p32.vz[i]};
        int ix, iy, iz;
        lead_cell(g, c, f, h, 10, d, ix, iy, iz);
        return cell_key(g, tab, ix, iy, iz, d);
    }
    return cell_key(g, tab, (int)p64.x[i], (int)p64.y[i], (int)p64.z[i], d);
}

// Warp-aggregated atomicAdd of 1 per lane on count[key], in two halves so a
// thread can have several in flight: agg_issue groups the lanes by key and lets
// each group's leader add the group's size; agg_slot (after every issue the
// thread has in flight) broadcasts the leader's old count and returns this
// lane's slot.
struct Agg {
    unsigned peers;
    int leader;
    uint32_t base;
};

__device__ __forceinline__ void agg_issue(uint32_t *count, uint32_t key, bool active, Agg &a)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned act = __ballot_sync(kFull, active);
    const uint32_t k = active ? key : 0xffffffffu - lane;
    a.peers = __match_any_sync(kFull, k) & act;
    a.leader = a.peers ? __ffs(a.peers) - 1 : -1;
    a.base = 0;
    if (active && (int)lane == a.leader) a.base = atomicAdd(count + key, (uint32_t)__popc(a.peers));
}

__device__ __forceinline__ uint32_t agg_slot(const Agg &a)
{
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t base = __shfl_sync(kFull, a.base, a.leader < 0 ? (int)lane : a.leader);
    return base + (uint32_t)__popc(a.peers & ((1u << lane) - 1u));
}

__device__ __forceinline__ uint32_t aggregated_inc(uint32_t *count, uint32_t key, bool active)
{
    Agg a;
    agg_issue(count, key, active, a);
    return agg_slot(a);
}

// Histogram add of 1 per active lane, one atomic per run of adjacent lanes with
// equal keys.  Lanes hold consecutive particles and the particles are mostly in
// cell order, so a warp holds a few runs; out-of-order keys just make more runs.
__device__ __forceinline__ void run_count(uint32_t *count, uint32_t key, bool active)
{
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t k = active ? key : 0xffffffffu - lane;   // inactive lanes end every run
    const uint32_t prev = __shfl_up_sync(kFull, k, 1);
    const bool head = lane == 0 || k != prev;
    const unsigned heads = __ballot_sync(kFull, head);
    const unsigned after = heads & ~((2u << lane) - 1u);   // run heads strictly after this lane
    const unsigned end = after ? (unsigned)__ffs(after) - 1u : 32u;
    if (active && head) atomicAdd(count + key, end - lane);
}

// The sort kernels are bound by memory latency (a cell load, then an atomic, then
// the record), so each thread keeps several independent particles in flight:
// four per iteration in the histogram; in the FP32 scatter four, whose record
// loads are all issued first and whose cursor atomics are all in flight before
// the first result is used (two in the FP64 scatter).  Launch bounds keep enough
// warps resident: five CTAs of 256 per SM for the histogram, three for the FP32
// scatter.
template <bool F32, bool LEAD = false>
__global__ void __launch_bounds__(256, 5) k_hist(Geom g, const uint32_t *tab, PartF64 p64, PartF32 p32, int64_t seg, int64_t n,
                       uint32_t *count, float h, DevDiag *d)
{
    static_assert(F32 || !LEAD, "sort lead: FP32 form");
    constexpr int U = LEAD ? 2 : 4;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += U * stride) {
        uint32_t key[U];
        bool act[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t i = base + u * stride + threadIdx.x;
            act[u] = i < n;
            key[u] = act[u] ? particle_key<F32>(g, tab, p64, p32, seg + i, LEAD ? h : 0.f, d) : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) run_count(count, key[u], act[u]);
    }
}

// One particle's record in registers.
template <bool F32>
struct Rec {
    double a[6];      // FP64 form: x, y, z, vx, vy, vz
    int32_t cell;     // FP32 form: packed cell, then offsets and velocities in f[]
    float f[6];
    uint32_t id;
};

template <bool F32>
__device__ __forceinline__ void rec_load(const PartF64 &s64, const PartF32 &s32, const uint32_t *sid, int64_t i,
                                         Rec<F32> &r)
{
    if (F32) {
        r.cell = s32.cell[i];
        r.f[0] = s32.ox[i]; r.f[1] = s32.oy[i]; r.f[2] = s32.oz[i];
        r.f[3] = s32.vx[i]; r.f[4] = s32.vy[i]; r.f[5] = s32.vz[i];
    } else {
        r.a[0] = s64.x[i]; r.a[1] = s64.y[i]; r.a[2] = s64.z[i];
        r.a[3] = s64.vx[i]; r.a[4] = s64.vy[i]; r.a[5] = s64.vz[i];
    }
    r.id = sid ? sid[i] : 0u;
}

template <bool F32>
__device__ __forceinline__ uint32_t rec_key(const Geom &g, const uint32_t *tab, const Rec<F32> &r, float h,
                                            DevDiag *d)
{
    if (F32) {
        if (h == 0.f) return cell_key(g, tab, cell_x(r.cell), cell_y(r.cell), cell_z(r.cell), d);
        int ix, iy, iz;
        lead_cell(g, r.cell, r.f, h, 10, d, ix, iy, iz);
        return cell_key(g, tab, ix, iy, iz, d);
    }
    return cell_key(g, tab, (int)r.a[0], (int)r.a[1], (int)r.a[2], d);
}

// FP32 form: the scatter writes each particle as one 32-byte record (cell, three
// offsets, three velocities, id) -- a whole L2 sector.  Once particles have
// drifted across tiles, a destination cell's slots are filled from source ranges
// megabytes apart, so per-array 4-byte scatters would leave sectors partly
// written when L2 evicts them (each costing a read-modify-write of the sector in
// HBM); whole-sector records never do.  A sequential pass then transposes the
// records back into the word arrays.
__device__ __forceinline__ void rec32_store(int4 *rec, int64_t j, const Rec<true> &r)
{
    rec[2 * j] = make_int4(r.cell, __float_as_int(r.f[0]), __float_as_int(r.f[1]), __float_as_int(r.f[2]));
    rec[2 * j + 1] = make_int4(__float_as_int(r.f[3]), __float_as_int(r.f[4]), __float_as_int(r.f[5]), (int)r.id);
}

__global__ void __launch_bounds__(256, 4) k_scatter_rec32(Geom g, const uint32_t *tab, PartF32 s32, const uint32_t *sid, int4 *rec,
                                int64_t seg, int64_t n, const uint32_t *start, uint32_t *cursor, float h,
                                DevDiag *d)
{
    constexpr int U = 2;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += U * stride) {
        Rec<true> r[U];
        bool act[U];
        uint32_t key[U], slot[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t i = base + u * stride + threadIdx.x;
            act[u] = i < n;
            if (act[u]) rec_load<true>(PartF64{}, s32, sid, seg + i, r[u]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) key[u] = act[u] ? rec_key<true>(g, tab, r[u], h, d) : 0u;
        Agg agg[U];
#pragma unroll
        for (int u = 0; u < U; ++u) agg_issue(cursor, key[u], act[u], agg[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) slot[u] = agg_slot(agg[u]);
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (act[u]) rec32_store(rec, seg + (int64_t)start[key[u]] + slot[u], r[u]);
    }
}

// Records [seg, seg + n) back into the word arrays (ids only when tracked).
__global__ void k_rec32_to_soa(const int4 *rec, int64_t seg, int64_t n, PartF32 p, uint32_t *ids)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        const int64_t j = seg + i;
        const int4 a = rec[2 * j], b = rec[2 * j + 1];
        p.cell[j] = a.x;
        p.ox[j] = __int_as_float(a.y); p.oy[j] = __int_as_float(a.z); p.oz[j] = __int_as_float(a.w);
        p.vx[j] = __int_as_float(b.x); p.vy[j] = __int_as_float(b.y); p.vz[j] = __int_as_float(b.z);
        if (ids) ids[j] = (uint32_t)b.w;
    }
}

// FP64 form: one 64-byte record per particle (positions, velocities, id,
// padding), two whole sectors, for the same reason.
__device__ __forceinline__ void rec64_store(double2 *rec, int64_t j, const Rec<false> &r)
{
    rec[4 * j] = make_double2(r.a[0], r.a[1]);
    rec[4 * j + 1] = make_double2(r.a[2], r.a[3]);
    rec[4 * j + 2] = make_double2(r.a[4], r.a[5]);
    rec[4 * j + 3] = make_double2(__longlong_as_double((long long)r.id), 0.0);
}

__global__ void k_scatter_rec64(Geom g, const uint32_t *tab, PartF64 s64, const uint32_t *sid, double2 *rec,
                                int64_t seg, int64_t n, const uint32_t *start, uint32_t *cursor, DevDiag *d)
{
    constexpr int U = 2;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n; base += U * stride) {
        Rec<false> r[U];
        bool act[U];
        uint32_t key[U], slot[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t i = base + u * stride + threadIdx.x;
            act[u] = i < n;
            if (act[u]) rec_load<false>(s64, PartF32{}, sid, seg + i, r[u]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) key[u] = act[u] ? rec_key<false>(g, tab, r[u], 0.f, d) : 0u;
#pragma unroll
        for (int u = 0; u < U; ++u) slot[u] = aggregated_inc(cursor, key[u], act[u]);
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (act[u]) rec64_store(rec, seg + (int64_t)start[key[u]] + slot[u], r[u]);
    }
}

__global__ void k_rec64_to_soa(const double2 *rec, int64_t seg, int64_t n, PartF64 p, uint32_t *ids)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
        const int64_t j = seg + i;
        const double2 a = rec[4 * j], b = rec[4 * j + 1], c = rec[4 * j + 2];
        p.x[j] = a.x; p.y[j] = a.y; p.z[j] = b.x;
        p.vx[j] = b.y; p.vy[j] = c.x; p.vz[j] = c.y;
        if (ids) ids[j] = (uint32_t)__double_as_longlong(rec[4 * j + 3].x);
    }
}

// ---- tile-local sort: the re-sort of particles that are already tile-sorted ----
//
// Between two sorts a particle moves a few cells, so most of a tile's particles
// (its source range from the last sort) still belong to that tile.  One CTA per
// source tile counts and places those "stayers" with shared-memory counters
// over the tile's cells; only the particles that now belong to another tile
// ("immigrants" there) use global counters.  Each cell's range starts with its
// stayers, then its immigrants: stay[key] is the stayer count, imm[key] the
// immigrant count (then the immigrant cursor).  Counters are bumped once per run
// of adjacent lanes with equal keys, and a run's lanes take consecutive slots in
// lane order, as in the global sort.

// One counter bump per run of adjacent lanes with equal keys.  The run's head
// adds the run length to the cell's counter (shared when the cell is in this
// CTA's tile, global otherwise); the returned value is the run's first slot
// once tile_run_slot() has broadcast it.
struct RunBump {
    uint32_t base;
    int head;   // lane of this lane's run head
};

__device__ __forceinline__ RunBump tile_run_bump(uint32_t *sh, uint32_t *gl, uint32_t key, uint32_t k0, uint32_t C,
                                                 bool active)
{
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t k = active ? key : 0xffffffffu - lane;   // inactive lanes end every run
    const uint32_t prev = __shfl_up_sync(kFull, k, 1);
    const bool head = lane == 0 || k != prev;
    const unsigned heads = __ballot_sync(kFull, head);
    const unsigned after = heads & ~((2u << lane) - 1u);   // run heads strictly after this lane
    const unsigned end = after ? (unsigned)__ffs(after) - 1u : 32u;
    RunBump r;
    r.base = 0;
    r.head = 31 - __clz(heads & ((2u << lane) - 1u));
    if (active && head) {
        const uint32_t local = key - k0;
        r.base = local < C ? atomicAdd(sh + local, end - lane) : atomicAdd(gl + key, end - lane);
    }
    return r;
}

__device__ __forceinline__ uint32_t tile_run_slot(const RunBump &r)
{
    const unsigned lane = threadIdx.x & 31u;
    return __shfl_sync(kFull, r.base, r.head) + (lane - (unsigned)r.head);
}

// The per-axis key table in shared memory: each CTA of a tile kernel copies it
// once, and every particle's three lookups are then shared loads instead of
// dependent global ones.
__device__ __forceinline__ uint32_t *stage_key_table(const Geom &g, const uint32_t *tab, uint32_t *dst)
{
    const int nt = g.nx + g.ny + g.nz;
    for (int i = threadIdx.x; i < nt; i += blockDim.x) dst[i] = __ldg(tab + i);
    return dst;
}

// The same key from the staged table, after the lead h (FP32 form).
__device__ __forceinline__ uint32_t shared_key_lead(const Geom &g, const uint32_t *stab, int32_t c, const float f[6],
                                                    float h, DevDiag *d)
{
    int ix, iy, iz;
    lead_cell(g, c, f, h, 11, d, ix, iy, iz);
    return stab[ix] + stab[g.nx + iy] + stab[g.nx + g.ny + iz];
}

__device__ __forceinline__ uint32_t shared_key(const Geom &g, const uint32_t *stab, int32_t c, DevDiag *d)
{
    int ix = cell_x(c), iy = cell_y(c), iz = cell_z(c);
    if ((unsigned)ix >= (unsigned)g.nx || (unsigned)iy >= (unsigned)g.ny || (unsigned)iz >= (unsigned)g.nz) {
        if (atomicCAS(&d->err_code, 0, OHPIC_ERR_BOUNDS) == 0) d->err_info = 11;
        ix = iy = iz = 0;
    }
    return stab[ix] + stab[g.nx + iy] + stab[g.nx + g.ny + iz];
}

template <bool F32>
__device__ __forceinline__ uint32_t shared_key_xyz(const Geom &g, const uint32_t *stab, double x, double y,
                                                   double z, DevDiag *d)
{
    int ix = (int)x, iy = (int)y, iz = (int)z;
    if ((unsigned)ix >= (unsigned)g.nx || (unsigned)iy >= (unsigned)g.ny || (unsigned)iz >= (unsigned)g.nz) {
        if (atomicCAS(&d->err_code, 0, OHPIC_ERR_BOUNDS) == 0) d->err_info = 11;
        ix = iy = iz = 0;
    }
    return stab[ix] + stab[g.nx + iy] + stab[g.nx + g.ny + iz];
}

// Counts of source tile blockIdx.x: stay[] for the tile's own cells (plain
// stores: every cell of every tile is written), imm[] (zeroed by the caller) by
// global atomics.
// LEAD (FP32 form): keys after the sort lead h, from the offsets and velocities
// as well as the cell.  The lead histogram fits 46 registers, so five CTAs per
// SM hide more of its load latency.
template <bool F32, bool LEAD = false>
__global__ void __launch_bounds__(256, LEAD ? 5 : 4) k_hist_tile(Geom g, const uint32_t *tab, PartF64 p64, PartF32 p32,
                                                   const int64_t *tb, uint32_t *stay, uint32_t *imm, float h,
                                                   DevDiag *d)
{
    static_assert(F32 || !LEAD, "sort lead: FP32 form");
    extern __shared__ uint32_t sh[];
    constexpr int U = F32 && !LEAD ? 8 : 4;
    const uint32_t C = (uint32_t)g.tile_cells, k0 = (uint32_t)blockIdx.x * C;
    for (uint32_t i = threadIdx.x; i < C; i += blockDim.x) sh[i] = 0u;
    const uint32_t *stab = stage_key_table(g, tab, sh + C);
    __syncthreads();
    const int64_t lo = tb[blockIdx.x], hi = tb[blockIdx.x + 1];
    for (int64_t base = lo; base < hi; base += U * (int64_t)blockDim.x) {
        uint32_t key[U];
        bool act[U];
        if constexpr (LEAD) {
            int32_t cell[U];
            float f[U][6];
#pragma unroll
            for (int u = 0; u < U; ++u) {   // every load of the iteration first
                const int64_t i = base + u * (int64_t)blockDim.x + threadIdx.x;
                act[u] = i < hi;
                cell[u] = act[u] ? p32.cell[i] : 0;
                f[u][0] = act[u] ? p32.ox[i] : 0.f;
                f[u][1] = act[u] ? p32.oy[i] : 0.f;
                f[u][2] = act[u] ? p32.oz[i] : 0.f;
                f[u][3] = act[u] ? p32.vx[i] : 0.f;
                f[u][4] = act[u] ? p32.vy[i] : 0.f;
                f[u][5] = act[u] ? p32.vz[i] : 0.f;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) key[u] = act[u] ? shared_key_lead(g, stab, cell[u], f[u], h, d) : 0u;
        } else if constexpr (F32) {
            int32_t cell[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {   // every load of the iteration first
                const int64_t i = base + u * (int64_t)blockDim.x + threadIdx.x;
                act[u] = i < hi;
                cell[u] = act[u] ? p32.cell[i] : 0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) key[u] = act[u] ? shared_key(g, stab, cell[u], d) : 0u;
        } else {
            double px[U], py[U], pz[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t i = base + u * (int64_t)blockDim.x + threadIdx.x;
                act[u] = i < hi;
                px[u] = act[u] ? p64.x[i] : 0.0;
                py[u] = act[u] ? p64.y[i] : 0.0;
                pz[u] = act[u] ? p64.z[i] : 0.0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) key[u] = act[u] ? shared_key_xyz<F32>(g, stab, px[u], py[u], pz[u], d) : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) tile_run_bump(sh, imm, key[u], k0, C, act[u]);
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < C; i += blockDim.x) stay[k0 + i] = sh[i];
}

// Scatter of source tile blockIdx.x into whole records: a stayer at
// start[key] + (its rank among the cell's stayers), an immigrant at
// start[key] + stay[key] + (its rank among the cell's immigrants; imm[] zeroed
// by the caller).  Two particles per thread per iteration, both counter bumps in
// flight before either slot is used.  (Six CTAs per SM, at 40 registers, made
// the electrons' scatter slower: 11.5 against 10.6 ms at 256^3.)
template <bool F32>
__global__ void __launch_bounds__(256, 4) k_scatter_tile(Geom g, const uint32_t *tab, PartF64 s64, PartF32 s32,
                                                         const uint32_t *sid, void *rec, const int64_t *tb,
                                                         int64_t seg, const uint32_t *start, const uint32_t *stay,
                                                         uint32_t *imm, float h, DevDiag *d)
{
    extern __shared__ uint32_t sh[];
    constexpr int U = 2;
    const uint32_t C = (uint32_t)g.tile_cells, k0 = (uint32_t)blockIdx.x * C;
    for (uint32_t i = threadIdx.x; i < C; i += blockDim.x) sh[i] = 0u;
    const uint32_t *stab = stage_key_table(g, tab, sh + C);
    __syncthreads();
    const int64_t lo = tb[blockIdx.x], hi = tb[blockIdx.x + 1];
    for (int64_t base = lo; base < hi; base += U * (int64_t)blockDim.x) {
        Rec<F32> r[U];
        bool act[U];
        uint32_t key[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t i = base + u * (int64_t)blockDim.x + threadIdx.x;
            act[u] = i < hi;
            if (act[u]) rec_load<F32>(s64, s32, sid, i, r[u]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if constexpr (F32)
                key[u] = act[u] ? (h != 0.f ? shared_key_lead(g, stab, r[u].cell, r[u].f, h, d)
                                            : shared_key(g, stab, r[u].cell, d))
                                : 0u;
            else key[u] = act[u] ? shared_key_xyz<F32>(g, stab, r[u].a[0], r[u].a[1], r[u].a[2], d) : 0u;
        }
        RunBump b[U];
#pragma unroll
        for (int u = 0; u < U; ++u) b[u] = tile_run_bump(sh, imm, key[u], k0, C, act[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t slot = tile_run_slot(b[u]);
            if (act[u]) {
                const bool own = key[u] - k0 < C;
                const int64_t j = seg + (int64_t)start[key[u]] + slot + (own ? 0u : stay[key[u]]);
                if constexpr (F32) rec32_store((int4 *)rec, j, r[u]);
                else rec64_store((double2 *)rec, j, r[u]);
            }
        }
    }
}

// Exclusive scan of one block of kScanBlock values; block total -> sums[blockIdx].
// in2, when given, is added to in element by element (the tile sort's stayer
// and immigrant counts).
__global__ void __launch_bounds__(kScanThreads) k_scan_block(const uint32_t *in, const uint32_t *in2, uint32_t *out,
                                                             int64_t n, uint32_t *sums)
{
    __shared__ uint32_t warp_tot[kScanThreads / 32];
    const int64_t b0 = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t local = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = b0 + k;
        v[k] = i < n ? in[i] + (in2 ? in2[i] : 0u) : 0u;
        local += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_tot[lane];
        uint32_t wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, wi, o);
            if (lane >= o) wi += t;
        }
        warp_tot[lane] = wi - w;   // exclusive warp offsets
        if (lane == 31 && sums) sums[blockIdx.x] = wi;
    }
    __syncthreads();
    uint32_t run = warp_tot[warp] + incl - local;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = b0 + k;
        if (i < n) out[i] = run;
        run += v[k];
    }
}

__global__ void k_add_offsets(uint32_t *out, int64_t n, const uint32_t *offs)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += offs[i / kScanBlock];
}

__global__ void k_tile_begin(Geom g, const uint32_t *start, int64_t seg, int64_t count, int64_t *tb)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < g.ntile) tb[t] = seg + (int64_t)start[t * g.tile_cells];
    if (t == g.ntile) tb[t] = seg + count;
}

// Exclusive scan of n values (in [+ in2] -> out) using tmp for the block sums of
// every level; returns the number of launches.
int scan_levels(cudaStream_t st, const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp,
                const uint32_t *in2 = nullptr)
{
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb <= 1) {
        k_scan_block<<<1, kScanThreads, 0, st>>>(in, in2, out, n, nullptr);
        return 1;
    }
    uint32_t *sums = tmp, *sums_scan = tmp + nb;
    k_scan_block<<<(unsigned)nb, kScanThreads, 0, st>>>(in, in2, out, n, sums);
    const int inner = scan_levels(st, sums, sums_scan, nb, tmp + 2 * nb);
    k_add_offsets<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, sums_scan);
    return inner + 2;
}

void scan_exclusive(ohpic_ctx *c, const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp,
                    const uint32_t *in2 = nullptr)
{
    c->launches += scan_levels(c->stream, in, out, n, tmp, in2);
}

// ---- multi-run sort: every (run, species) segment in one pass per stage ----

// Loads the inclusive chunk prefix into shared memory; returns the chunk total.
__device__ __forceinline__ int32_t load_chunk_ends(const MultiSort &m, int32_t *s_end, int nseg)
{
    for (int i = threadIdx.x; i < nseg; i += blockDim.x) s_end[i] = m.chunk_end[i];
    __syncthreads();
    return nseg > 0 ? s_end[nseg - 1] : 0;
}

__device__ __forceinline__ int find_seg(const int32_t *s_end, int nseg, int64_t chunk)
{
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if ((int64_t)s_end[mid] > chunk) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

__global__ void k_hist_multi(MultiSort m)
{
    __shared__ int32_t s_end[kMaxSortSegs];
    const int nseg = *m.nseg;
    const int32_t total = load_chunk_ends(m, s_end, nseg);
    for (int64_t c = blockIdx.x; c < total; c += gridDim.x) {
        const int si = find_seg(s_end, nseg, c);
        const SortSeg &sg = m.segs[si];
        const int64_t first = (c - (si > 0 ? s_end[si - 1] : 0)) * (int64_t)kSortChunk;
        const int64_t last = min(first + (int64_t)kSortChunk, sg.count);
        for (int64_t base = first; base < last; base += blockDim.x) {
            const int64_t i = base + threadIdx.x;
            const bool active = i < last;
            const uint32_t key = active ? particle_key<true>(sg.g, nullptr, PartF64{}, sg.p, sg.off + i, sg.h, sg.diag) : 0u;
            aggregated_inc(m.count + sg.key_base, key, active);
        }
    }
}

// Scatter of every segment into its run's record area (whole 32-byte records,
// as in the single-context FP32 sort), then the records back into the arrays.
__global__ void k_scatter_multi(MultiSort m)
{
    __shared__ int32_t s_end[kMaxSortSegs];
    const int nseg = *m.nseg;
    const int32_t total = load_chunk_ends(m, s_end, nseg);
    for (int64_t c = blockIdx.x; c < total; c += gridDim.x) {
        const int si = find_seg(s_end, nseg, c);
        const SortSeg &sg = m.segs[si];
        const int64_t first = (c - (si > 0 ? s_end[si - 1] : 0)) * (int64_t)kSortChunk;
        const int64_t last = min(first + (int64_t)kSortChunk, sg.count);
        const uint32_t base0 = m.start[sg.key_base];
        for (int64_t base = first; base < last; base += blockDim.x) {
            const int64_t i = base + threadIdx.x;
            const bool active = i < last;
            Rec<true> r;
            if (active) rec_load<true>(PartF64{}, sg.p, sg.ids, sg.off + i, r);
            const uint32_t key = active ? rec_key<true>(sg.g, nullptr, r, sg.h, sg.diag) : 0u;
            const uint32_t slot = aggregated_inc(m.cursor + sg.key_base, key, active);
            if (active) rec32_store(sg.rec, sg.off + (int64_t)(m.start[sg.key_base + key] - base0) + slot, r);
        }
    }
}

__global__ void k_rec32_to_soa_multi(MultiSort m)
{
    __shared__ int32_t s_end[kMaxSortSegs];
    const int nseg = *m.nseg;
    const int32_t total = load_chunk_ends(m, s_end, nseg);
    for (int64_t c = blockIdx.x; c < total; c += gridDim.x) {
        const int si = find_seg(s_end, nseg, c);
        const SortSeg &sg = m.segs[si];
        const int64_t first = (c - (si > 0 ? s_end[si - 1] : 0)) * (int64_t)kSortChunk;
        const int64_t last = min(first + (int64_t)kSortChunk, sg.count);
        for (int64_t i = first + threadIdx.x; i < last; i += blockDim.x) {
            const int64_t j = sg.off + i;
            const int4 a = sg.rec[2 * j], b = sg.rec[2 * j + 1];
            sg.p.cell[j] = a.x;
            sg.p.ox[j] = __int_as_float(a.y); sg.p.oy[j] = __int_as_float(a.z); sg.p.oz[j] = __int_as_float(a.w);
            sg.p.vx[j] = __int_as_float(b.x); sg.p.vy[j] = __int_as_float(b.y); sg.p.vz[j] = __int_as_float(b.z);
            if (sg.ids) sg.ids[j] = (uint32_t)b.w;
        }
    }
}

// tile_begin of every segment: blockIdx.y = segment.
__global__ void k_tile_begin_multi(MultiSort m)
{
    if ((int)blockIdx.y >= *m.nseg) return;
    const SortSeg &sg = m.segs[blockIdx.y];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nt = sg.g.ntile;
    if (t > nt) return;
    const uint32_t base0 = m.start[sg.key_base];
    sg.tile_begin[t] = t == nt ? sg.off + sg.count
                               : sg.off + (int64_t)(m.start[sg.key_base + t * sg.g.tile_cells] - base0);
}

int grid_of(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    return b < 1 ? 1 : (int)b;
}

}  // namespace

int64_t scan_tmp_elems(int64_t n)
{
    int64_t total = 0;
    for (int64_t m = n; m > kScanBlock;) {
        const int64_t nb = (m + kScanBlock - 1) / kScanBlock;
        total += 2 * nb;
        m = nb;
    }
    return total + 16;
}

int scan_u32(cudaStream_t st, const uint32_t *in, uint32_t *out, int64_t n, uint32_t *tmp)
{
    return scan_levels(st, in, out, n, tmp);
}

int launch_sort_hist_multi(cudaStream_t st, const MultiSort &m, int64_t chunks)
{
    if (chunks <= 0) return 0;
    const int64_t grid = chunks < 152 * 8 ? chunks : 152 * 8;
    k_hist_multi<<<(unsigned)grid, 256, 0, st>>>(m);
    return 1;
}

// Scan of the key space, tile starts, then the scatter (the cursor array must be
// zero; the caller clears it before this call).
int launch_sort_finish_multi(cudaStream_t st, const MultiSort &m, int64_t chunks, int64_t max_ntile,
                             int max_seg, int64_t nkeys, uint32_t *scan_tmp)
{
    int launches = scan_levels(st, m.count, m.start, nkeys, scan_tmp);
    if (max_seg > 0) {
        dim3 grid((unsigned)((max_ntile + 1 + 255) / 256), (unsigned)max_seg);
        k_tile_begin_multi<<<grid, 256, 0, st>>>(m);
        ++launches;
    }
    if (chunks > 0) {
        const int64_t grid = chunks < 152 * 8 ? chunks : 152 * 8;
        k_scatter_multi<<<(unsigned)grid, 256, 0, st>>>(m);
        k_rec32_to_soa_multi<<<(unsigned)grid, 256, 0, st>>>(m);
        launches += 2;
    }
    return launches;
}

void materialize_records(ohpic_ctx *c)
{
    if (!c->rec_pending) return;
    const int4 *rec = (const int4 *)c->pblock[1 - c->cur];
    for (int s = 0; s < c->cfg.nspecies; ++s) {
        const int64_t n = c->count[s];
        if (n <= 0) continue;
        k_rec32_to_soa<<<grid_of(n), 256, 0, c->stream>>>(rec, c->seg[s], n, c->p32[c->cur], c->ids[c->cur]);
        ++c->launches;
    }
    c->rec_pending = false;
}

// Shared memory of the tile-local re-sort (the tile's counters and the key table)
// stays within the default 48 KB per CTA.
constexpr size_t kTileSortMaxShared = 48 * 1024;

// Re-sort of particles already sorted on the current tiling (tile_begin valid):
// per species, tile-local counts, the scan of stayers + immigrants, tile starts,
// then the tile-local scatter into records (FP32: left for the next push; FP64:
// transposed back here).
static void sort_tiles(ohpic_ctx *c, float h)
{
    const Geom &g = c->g;
    const bool f32 = c->cfg.precision == OHPIC_FP32;
    const int src = c->cur, dst = 1 - c->cur;
    const size_t smem = sizeof(uint32_t) * ((size_t)g.tile_cells + g.nx + g.ny + g.nz);
    for (int s = 0; s < c->cfg.nspecies; ++s) {
        const int64_t n = c->count[s];
        int64_t *tb = c->tile_begin + (int64_t)s * (g.ntile + 1);
        cudaMemsetAsync(c->cell_count, 0, sizeof(uint32_t) * g.ncell, c->stream);
        if (f32 && h != 0.f)
            k_hist_tile<true, true><<<(unsigned)g.ntile, 256, smem, c->stream>>>(
                g, c->key_table, c->p64[src], c->p32[src], tb, c->cell_stay, c->cell_count, h, c->diag);
        else if (f32)
            k_hist_tile<true><<<(unsigned)g.ntile, 256, smem, c->stream>>>(g, c->key_table, c->p64[src], c->p32[src],
                                                                          tb, c->cell_stay, c->cell_count, 0.f,
                                                                          c->diag);
        else
            k_hist_tile<false><<<(unsigned)g.ntile, 256, smem, c->stream>>>(g, c->key_table, c->p64[src], c->p32[src],
                                                                           tb, c->cell_stay, c->cell_count, 0.f,
                                                                           c->diag);
        ++c->launches;
        scan_exclusive(c, c->cell_stay, c->cell_start, g.ncell, c->scan_tmp, c->cell_count);
        cudaMemsetAsync(c->cell_count, 0, sizeof(uint32_t) * g.ncell, c->stream);
        if (f32) {
            k_scatter_tile<true><<<(unsigned)g.ntile, 256, smem, c->stream>>>(
                g, c->key_table, c->p64[src], c->p32[src], c->ids[src], c->pblock[dst], tb, c->seg[s], c->cell_start,
                c->cell_stay, c->cell_count, h, c->diag);
            ++c->launches;
            c->rec_pending = true;
        } else {
            double2 *rec = (double2 *)c->pblock[dst];
            k_scatter_tile<false><<<(unsigned)g.ntile, 256, smem, c->stream>>>(
                g, c->key_table, c->p64[src], c->p32[src], c->ids[src], rec, tb, c->seg[s], c->cell_start,
                c->cell_stay, c->cell_count, 0.f, c->diag);
            k_rec64_to_soa<<<grid_of(n), 256, 0, c->stream>>>(rec, c->seg[s], n, c->p64[src], c->ids[src]);
            c->launches += 2;
        }
        // the new tile starts, after the scatter has read the old ones
        k_tile_begin<<<(unsigned)((g.ntile + 1 + 255) / 256), 256, 0, c->stream>>>(g, c->cell_start, c->seg[s], n,
                                                                                    tb);
        ++c->launches;
    }
}

int sort_particles(ohpic_ctx *c)
{
    const Geom &g = c->g;
    const bool f32 = c->cfg.precision == OHPIC_FP32;
    const int src = c->cur, dst = 1 - c->cur;   // the records come back into the current buffer
    materialize_records(c);
    const int axes = g.nx + g.ny + g.nz;
    k_key_table<<<(unsigned)((axes + 255) / 256), 256, 0, c->stream>>>(g, c->key_table);
    ++c->launches;
    // the lead in cells per unit velocity: sort_lead steps of the last step's dt
    // (the configured dt before the first step)
    const double dt = std::isfinite(c->sc_dt) ? c->sc_dt : c->cfg.dt;
    float h = f32 && c->sort_lead > 0 ? (float)(c->sort_lead * dt) : 0.f;
    if (!std::isfinite(h)) h = 0.f;   // no usable step yet: sort by the current cell
    if (c->sorted && sizeof(uint32_t) * ((size_t)g.tile_cells + axes) <= kTileSortMaxShared) {
        sort_tiles(c, h);
        c->steps_since_sort = 0;
        return OHPIC_OK;
    }
    for (int s = 0; s < c->cfg.nspecies; ++s) {
        const int64_t n = c->count[s];
        int64_t *tb = c->tile_begin + (int64_t)s * (g.ntile + 1);
        cudaMemsetAsync(c->cell_count, 0, sizeof(uint32_t) * g.ncell, c->stream);
        if (n > 0) {
            if (f32)
                if (h != 0.f)
                    k_hist<true, true><<<grid_of(n), 256, 0, c->stream>>>(g, c->key_table, c->p64[src],
                                                                          c->p32[src], c->seg[s], n, c->cell_count,
                                                                          h, c->diag);
                else
                    k_hist<true><<<grid_of(n), 256, 0, c->stream>>>(g, c->key_table, c->p64[src], c->p32[src],
                                                                    c->seg[s], n, c->cell_count, 0.f, c->diag);
            else
                k_hist<false><<<grid_of(n), 256, 0, c->stream>>>(g, c->key_table, c->p64[src], c->p32[src],
                                                                 c->seg[s], n, c->cell_count, 0.f, c->diag);
            ++c->launches;
        }
        scan_exclusive(c, c->cell_count, c->cell_start, g.ncell, c->scan_tmp);
        k_tile_begin<<<(unsigned)((g.ntile + 1 + 255) / 256), 256, 0, c->stream>>>(g, c->cell_start, c->seg[s], n,
                                                                                    tb);
        ++c->launches;
        if (n > 0) {
            cudaMemsetAsync(c->cell_count, 0, sizeof(uint32_t) * g.ncell, c->stream);
            // records in the other buffer's block, then back into this buffer:
            // FP32 by the next push (or materialize_records), FP64 here
            if (f32) {
                int4 *rec = (int4 *)c->pblock[dst];
                k_scatter_rec32<<<grid_of(n), 256, 0, c->stream>>>(g, c->key_table, c->p32[src], c->ids[src], rec,
                                                                   c->seg[s], n, c->cell_start, c->cell_count, h,
                                                                   c->diag);
                ++c->launches;
                c->rec_pending = true;
            } else {
                double2 *rec = (double2 *)c->pblock[dst];
                k_scatter_rec64<<<grid_of(n), 256, 0, c->stream>>>(g, c->key_table, c->p64[src], c->ids[src], rec,
                                                                   c->seg[s], n, c->cell_start, c->cell_count,
                                                                   c->diag);
                k_rec64_to_soa<<<grid_of(n), 256, 0, c->stream>>>(rec, c->seg[s], n, c->p64[src], c->ids[src]);
                c->launches += 2;
            }
        }
    }
    c->sorted = true;
    c->steps_since_sort = 0;
    return OHPIC_OK;
}

}  // namespace ohpic
