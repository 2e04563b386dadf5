// push_f32.cu -- the FP32 precision form of the tiled particle kernels.
//
// Reference path (per particle, src/ohhelppic3d.f90:311-358):
//   scatter   src/scatter/linear_scatter.f90:32-53
//   interp    src/interpolator/linear_interpolator.f90:33-67
//   move      src/particle_mover/particle_mover_boris.f90:37-62
//   boundary  src/particle_boundary/periodic_particle_boundary.f90:42-53 (twice)
//
// Particle state: int32 packed cell (ix | iy<<11 | iz<<22), FP32 offsets in
// [0, 1) and FP32 velocities, 28 bytes per particle in 7 SoA arrays.
//
// Mapping.  Lane l of a warp handles four consecutive particles (base + 4l ..
// base + 4l + 3; two as a tunable), so the 32 lanes hold 128 consecutive
// particles of the cell-sorted order: their cells are mostly the same few, and
// the 8 node loads of the gather are shared-memory broadcasts.  Loads and stores
// are 16-byte vector accesses coalesced across the warp; the next quad is
// prefetched into shared memory while the current one is computed.
//
// Deposit in fixed point.  Each particle's 8 CIC weights are integers in units of
// 2^-24 that sum to exactly 2^24 (an exact axis-by-axis split; charge is
// conserved exactly).  A lane sums the weights of its consecutive same-cell
// particles in registers and adds them to a shared 64-bit box kept as 32-bit
// low/high words: 32-bit shared atomic adds are native, unlike FP32 shared
// atomics.  By default (OHPIC_DEPOSIT_LANES) the lanes add directly; warp
// combinations before the add (segmented shuffles over runs of equal cells,
// hardware reduces) are tunable alternatives that measured slower with four
// particles per lane.  The box is flushed once per CTA into per-species 64-bit
// global sums.  All of it is integer addition, so the deposit does not depend on
// the order in which atomics land.
//
// After a cell sort.  The sort (sort.cu) leaves every particle as a 32-byte
// record in the second buffer; the next push (tiled_f32_rec) reads those
// records in place of the seven arrays and writes the arrays and the ids, so
// the sort has no transpose pass of its own.  The arithmetic is the same
// advance_pair(), so both pushes give the same bits.
#include <type_traits>

#include "tile_common.cuh"
#include "tma.cuh"

namespace ohpic {
namespace {

// The launch shape the autotuner picks for the dense plasmas (tile 16 x 8 x 8
// cells, halo 2) has its own push kernels with the box geometry fixed at
// compile time: node offsets become immediates of the shared-memory loads and
// atomics instead of registers and adds.
constexpr int kFixTx = 16, kFixTy = 8, kFixTz = 8, kFixHalo = 2;

// Segmented sum of u over runs of equal keys held by adjacent lanes (at most 5
// shuffle steps, stopping early when the runs are short); returns true in the
// run's first lane, which then holds the run total.
__device__ __forceinline__ bool run_sum(int key, unsigned u[8])
{
    const int lane = (int)(threadIdx.x & 31u);
    const int prev = __shfl_up_sync(kFull, key, 1);
    const bool head = lane == 0 || key != prev;
    const unsigned heads = __ballot_sync(kFull, head);
    const unsigned after = heads & ~((2u << lane) - 1u);   // run heads strictly after this lane
    const int run_end = after ? __ffs(after) - 2 : 31;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const bool take = lane + d <= run_end;
        if (!__any_sync(kFull, take)) break;
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const unsigned t = __shfl_down_sync(kFull, u[v], d);
            if (take) u[v] += t;
        }
    }
    return head;
}

// Deposit box: a node's weight sum (units of 2^-24) is the 64-bit value
// hi:lo kept in two 32-bit words; an add goes to lo with a native 32-bit
// shared atomic and a carry out of lo increments hi.
__device__ __forceinline__ void box_add8(unsigned *hi, unsigned *lo, int key, int sx, int sxy, const unsigned u[8])
{
    const int off[8] = {0, 1, sx, sx + 1, sxy, sxy + 1, sxy + sx, sxy + sx + 1};
    unsigned old[8];
#pragma unroll
    for (int v = 0; v < 8; ++v) old[v] = atomicAdd(lo + key + off[v], u[v]);
    // A carry needs old + u >= 2^32, so old or u at least 2^31: one test of the
    // words' OR rules carries out for all eight (node sums stay far below 2^31
    // units, 128 particle weights, in any plasma of sane density); past it the
    // eight high-word adds (of 0 or 1) go without a branch each.
    unsigned m = 0u;
#pragma unroll
    for (int v = 0; v < 8; ++v) m |= old[v] | u[v];
    if (m >> 31) {
#pragma unroll
        for (int v = 0; v < 8; ++v) atomicAdd(hi + key + off[v], (unsigned)(old[v] + u[v] < old[v]));
    }
}

// Adds u (weights, key = box index of the cell or < 0) to the shared box.  DEP
// picks how lanes that share a key are combined first (OHPIC_DEPOSIT_*): not at
// all (LANES); runs of adjacent lanes by shuffles; one hardware warp reduce when
// every lane holds the same key, else runs; or __match_any_sync groups reduced
// with __reduce_add_sync.  All 32 lanes must call this.
template <int DEP>
__device__ __forceinline__ void warp_run_deposit(int key, unsigned u[8], unsigned *lo, unsigned *hi, int sx,
                                                 int sxy)
{
    if (DEP == OHPIC_DEPOSIT_LANES) {
        if (key >= 0) box_add8(hi, lo, key, sx, sxy, u);
        return;
    }
    const unsigned lane = threadIdx.x & 31u;
    bool head;
    if (DEP == OHPIC_DEPOSIT_GROUPS) {
        // Cell-sorted particles put few distinct cells in a warp: reduce each of
        // the first three over the whole warp (redux.sync, all lanes converged),
        // the lanes left after that by runs.
        unsigned todo = __ballot_sync(kFull, key >= 0);
#pragma unroll 1
        for (int round = 0; round < 3 && todo; ++round) {
            const int leader = __ffs(todo) - 1;
            const int k = __shfl_sync(kFull, key, leader);
            const bool mine = key == k;
            unsigned s[8];
#pragma unroll
            for (int v = 0; v < 8; ++v) s[v] = __reduce_add_sync(kFull, mine ? u[v] : 0u);
            if ((int)lane == leader) box_add8(hi, lo, k, sx, sxy, s);
            todo &= ~__ballot_sync(kFull, mine);
        }
        if (!todo) return;
        if (!((todo >> lane) & 1u)) key = -1;
        head = run_sum(key, u);
    } else if (DEP == OHPIC_DEPOSIT_MATCH) {
        const unsigned peers = __match_any_sync(kFull, key);
        head = (peers & ((1u << lane) - 1u)) == 0u;
        if (peers != (1u << lane)) {
#pragma unroll
            for (int v = 0; v < 8; ++v) u[v] = __reduce_add_sync(peers, u[v]);
        }
    } else if (DEP == OHPIC_DEPOSIT_UNIFORM) {
        const int k0 = __shfl_sync(kFull, key, 0);
        if (__all_sync(kFull, key == k0)) {
#pragma unroll
            for (int v = 0; v < 8; ++v) u[v] = __reduce_add_sync(kFull, u[v]);
            head = lane == 0;
        } else {
            head = run_sum(key, u);
        }
    } else {
        head = run_sum(key, u);
    }
    if (head && key >= 0) box_add8(hi, lo, key, sx, sxy, u);
}

// Componentwise FP32 pair arithmetic.  GB300 issues each of these as one
// instruction for both components, and each component is rounded exactly as the
// scalar operation (__fmul_rn, __fadd_rn, __fmaf_rn): no contraction.  The push
// carries two particles through one instruction stream this way, so every
// particle's arithmetic is the same sequence of roundings whichever pair or lane
// it sits in.
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }
// 1 - r, rounded once (r * -1 is exact).
__device__ __forceinline__ float2 one_minus2(float2 r) { return __ffma2_rn(r, bc2(-1.f), bc2(1.f)); }

// CIC weights of nodes floor(x) and floor(x)+1 for a pair of offsets.
template <int CONV>
__device__ __forceinline__ void cic2(float2 r, float2 &w0, float2 &w1)
{
    if (CONV == OHPIC_WEIGHTS_REFERENCE) {
        w0 = r;
        w1 = one_minus2(r);
    } else {
        w0 = one_minus2(r);
        w1 = r;
    }
}

// CIC weights of one particle in units of 2^-24, summing to exactly 2^24.  The
// total is split exactly, one axis at a time: x into X1 = round(wx1 * 2^24) and
// X0 = 2^24 - X1, each half into y parts, each quarter into z parts.  A child is
// rounded from its parent's FP32 product and clamped to the parent's integer, the
// sibling is the difference, so every weight is non-negative and the eight add
// up to 2^24 with no fix-up pass (7 float-to-integer conversions instead of 8).
// The products come in for a pair of particles (component c of each argument).
// Y11 and Z11 need no clamp: f11 = fx1 * wy1 and z11 = f11 * wz1 with weights in
// [0, 1], and rounding is monotonic, so round(z11) <= round(f11) <= round(fx1).
__device__ __forceinline__ void split_weights(float fx1, float f11, float f01, float z00, float z10, float z01,
                                              float z11, unsigned u[8])
{
    const unsigned X1 = __float2uint_rn(fx1), X0 = (1u << 24) - X1;
    const unsigned Y11 = __float2uint_rn(f11), Y01 = min(__float2uint_rn(f01), X0);
    const unsigned Y10 = X1 - Y11, Y00 = X0 - Y01;
    const unsigned Z00 = min(__float2uint_rn(z00), Y00), Z10 = min(__float2uint_rn(z10), Y10);
    const unsigned Z01 = min(__float2uint_rn(z01), Y01), Z11 = __float2uint_rn(z11);
    u[0] = Y00 - Z00; u[1] = Y10 - Z10; u[2] = Y01 - Z01; u[3] = Y11 - Z11;
    u[4] = Z00; u[5] = Z10; u[6] = Z01; u[7] = Z11;
}

template <int W>
__device__ __forceinline__ void fixed_weights2(float2 ox, float2 oy, float2 oz, unsigned u0[8], unsigned u1[8])
{
    float2 wx0, wx1, wy0, wy1, wz0, wz1;
    cic2<W>(ox, wx0, wx1);
    cic2<W>(oy, wy0, wy1);
    cic2<W>(oz, wz0, wz1);
    const float2 S = bc2(kWeightScale);
    const float2 fx1 = mul2(wx1, S), fx0 = mul2(wx0, S);   // exact: power-of-two scale
    const float2 f11 = mul2(fx1, wy1), f01 = mul2(fx0, wy1), f10 = mul2(fx1, wy0), f00 = mul2(fx0, wy0);
    const float2 z00 = mul2(f00, wz1), z10 = mul2(f10, wz1), z01 = mul2(f01, wz1), z11 = mul2(f11, wz1);
    split_weights(fx1.x, f11.x, f01.x, z00.x, z10.x, z01.x, z11.x, u0);
    split_weights(fx1.y, f11.y, f01.y, z00.y, z10.y, z01.y, z11.y, u1);
}

// Node indices in 32 bits: the packed cell limits the FP32 form's grid to 2^32
// nodes, so every index and partial sum fits an unsigned word.
__device__ __forceinline__ void deposit_global_fixed(const Geom &g, unsigned long long *w, int ix, int iy, int iz,
                                                     const unsigned u[8])
{
    const unsigned nx = (unsigned)g.nx, nxy = (unsigned)g.nx * (unsigned)g.ny;
    const unsigned x0 = (unsigned)ix, x1 = ix + 1 == g.nx ? 0u : (unsigned)ix + 1u;
    const unsigned y0 = (unsigned)iy * nx, y1 = (iy + 1 == g.ny ? 0u : (unsigned)iy + 1u) * nx;
    const unsigned z0 = (unsigned)iz * nxy, z1 = (iz + 1 == g.nz ? 0u : (unsigned)iz + 1u) * nxy;
    atomicAdd(w + (x0 + y0 + z0), (unsigned long long)u[0]);
    atomicAdd(w + (x1 + y0 + z0), (unsigned long long)u[1]);
    atomicAdd(w + (x0 + y1 + z0), (unsigned long long)u[2]);
    atomicAdd(w + (x1 + y1 + z0), (unsigned long long)u[3]);
    atomicAdd(w + (x0 + y0 + z1), (unsigned long long)u[4]);
    atomicAdd(w + (x1 + y0 + z1), (unsigned long long)u[5]);
    atomicAdd(w + (x0 + y1 + z1), (unsigned long long)u[6]);
    atomicAdd(w + (x1 + y1 + z1), (unsigned long long)u[7]);
}

// Shared box: E nodes (float4) then the low and high words of the weight sums.
__device__ __forceinline__ void stage_f32(const TileArgs &a, const Item &it, float4 *sE, unsigned *lo, unsigned *hi,
                                          bool need_e, bool need_w)
{
    // One box row (fixed y, z) per warp iteration, lanes along x.
    const Geom &g = a.g;
    if (need_e) {
        const float4 *E = (const float4 *)a.epad;
        const int rows = g.sy * g.sz, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
        for (int r = threadIdx.x >> 5; r < rows; r += nw) {
            const int cz = r / g.sy, by = r - cz * g.sy;
            // padded index of node x0 - halo + ax is x0 + ax
            const float4 *src = E + ((int64_t)(it.z0 + cz) * g.gy + (it.y0 + by)) * g.gx + it.x0;
            const int base = r * g.sx;
            for (int ax = lane; ax < g.sx; ax += 32) sE[base + ax] = __ldg(src + ax);
        }
    }
    if (need_w) {
        const int s3 = g.sx * g.sy * g.sz;
        for (int i = threadIdx.x; i < s3; i += blockDim.x) {
            lo[i] = 0u;
            hi[i] = 0u;
        }
    }
}

__device__ __forceinline__ void flush_f32(const TileArgs &a, const Item &it, const unsigned *lo, const unsigned *hi)
{
    const Geom &g = a.g;
    unsigned long long *w = a.wsum + (int64_t)it.sp * g.ncell;
    const int rows = g.sy * g.sz, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = threadIdx.x >> 5; r < rows; r += nw) {
        const int cz = r / g.sy, by = r - cz * g.sy;
        const int y = wrapi(it.y0 - g.halo + by, g.ny);
        const int z = wrapi(it.z0 - g.halo + cz, g.nz);
        unsigned long long *row = w + (int64_t)g.nx * (y + (int64_t)g.ny * z);
        const int base = r * g.sx;
        for (int ax = lane; ax < g.sx; ax += 32) {
            const unsigned long long v = ((unsigned long long)hi[base + ax] << 32) | lo[base + ax];
            if (v) {
                int x = it.x0 - g.halo + ax;
                if ((unsigned)x >= (unsigned)g.nx) x = wrapi(x, g.nx);
                atomicAdd(row + x, v);
            }
        }
    }
}

struct P32 {
    int32_t cell;
    float ox, oy, oz, vx, vy, vz;
};

// Particles 2g and 2g+1: one 8-byte vector per array.
template <bool kGather>
__device__ __forceinline__ void load_pair(const PartF32 &p, int64_t g, P32 r[2])
{
    const int2 c = *(const int2 *)(p.cell + 2 * g);
    const float2 x = *(const float2 *)(p.ox + 2 * g);
    const float2 y = *(const float2 *)(p.oy + 2 * g);
    const float2 z = *(const float2 *)(p.oz + 2 * g);
    r[0].cell = c.x; r[1].cell = c.y;
    r[0].ox = x.x; r[1].ox = x.y;
    r[0].oy = y.x; r[1].oy = y.y;
    r[0].oz = z.x; r[1].oz = z.y;
    if (kGather) {
        const float2 u = *(const float2 *)(p.vx + 2 * g);
        const float2 v = *(const float2 *)(p.vy + 2 * g);
        const float2 w = *(const float2 *)(p.vz + 2 * g);
        r[0].vx = u.x; r[1].vx = u.y;
        r[0].vy = v.x; r[1].vy = v.y;
        r[0].vz = w.x; r[1].vz = w.y;
    } else {
        r[0].vx = r[0].vy = r[0].vz = r[1].vx = r[1].vy = r[1].vz = 0.f;
    }
}

__device__ __forceinline__ void store_pair(const PartF32 &p, int64_t g, const P32 r[2])
{
    *(int2 *)(p.cell + 2 * g) = make_int2(r[0].cell, r[1].cell);
    *(float2 *)(p.ox + 2 * g) = make_float2(r[0].ox, r[1].ox);
    *(float2 *)(p.oy + 2 * g) = make_float2(r[0].oy, r[1].oy);
    *(float2 *)(p.oz + 2 * g) = make_float2(r[0].oz, r[1].oz);
    *(float2 *)(p.vx + 2 * g) = make_float2(r[0].vx, r[1].vx);
    *(float2 *)(p.vy + 2 * g) = make_float2(r[0].vy, r[1].vy);
    *(float2 *)(p.vz + 2 * g) = make_float2(r[0].vz, r[1].vz);
}

// Particles 4g .. 4g+3: one 16-byte vector per array.
template <bool kGather>
__device__ __forceinline__ void load_quad(const PartF32 &p, int64_t g, P32 r[4])
{
    const int4 c = *(const int4 *)(p.cell + 4 * g);
    const float4 x = *(const float4 *)(p.ox + 4 * g);
    const float4 y = *(const float4 *)(p.oy + 4 * g);
    const float4 z = *(const float4 *)(p.oz + 4 * g);
    r[0].cell = c.x; r[1].cell = c.y; r[2].cell = c.z; r[3].cell = c.w;
    r[0].ox = x.x; r[1].ox = x.y; r[2].ox = x.z; r[3].ox = x.w;
    r[0].oy = y.x; r[1].oy = y.y; r[2].oy = y.z; r[3].oy = y.w;
    r[0].oz = z.x; r[1].oz = z.y; r[2].oz = z.z; r[3].oz = z.w;
    if (kGather) {
        const float4 u = *(const float4 *)(p.vx + 4 * g);
        const float4 v = *(const float4 *)(p.vy + 4 * g);
        const float4 w = *(const float4 *)(p.vz + 4 * g);
        r[0].vx = u.x; r[1].vx = u.y; r[2].vx = u.z; r[3].vx = u.w;
        r[0].vy = v.x; r[1].vy = v.y; r[2].vy = v.z; r[3].vy = v.w;
        r[0].vz = w.x; r[1].vz = w.y; r[2].vz = w.z; r[3].vz = w.w;
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) r[j].vx = r[j].vy = r[j].vz = 0.f;
    }
}

// Prefetch of the next quad: 16-byte cp.async copies (one per array) into this
// thread's own slots of a shared stage, so the next iteration's loads are in
// flight during this one's arithmetic without holding registers.  The thread
// reads back only what it copied, after cp.async.wait_group, so no block-wide
// synchronisation is needed.  Slot of array k: st[k * blockDim.x + threadIdx.x].
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(smem_dst)), "l"(gsrc) : "memory");
}

template <bool kGather>
__device__ __forceinline__ void prefetch_quad(float4 *st, const PartF32 &p, int64_t g)
{
    const int n = blockDim.x, i = threadIdx.x;
    cp_async16(st + i, p.cell + 4 * g);
    cp_async16(st + n + i, p.ox + 4 * g);
    cp_async16(st + 2 * n + i, p.oy + 4 * g);
    cp_async16(st + 3 * n + i, p.oz + 4 * g);
    if (kGather) {
        cp_async16(st + 4 * n + i, p.vx + 4 * g);
        cp_async16(st + 5 * n + i, p.vy + 4 * g);
        cp_async16(st + 6 * n + i, p.vz + 4 * g);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

template <bool kGather>
__device__ __forceinline__ void read_quad(const float4 *st, P32 r[4])
{
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    const int n = blockDim.x, i = threadIdx.x;
    const float4 cf = st[i];
    const float4 x = st[n + i], y = st[2 * n + i], z = st[3 * n + i];
    r[0].cell = __float_as_int(cf.x); r[1].cell = __float_as_int(cf.y);
    r[2].cell = __float_as_int(cf.z); r[3].cell = __float_as_int(cf.w);
    r[0].ox = x.x; r[1].ox = x.y; r[2].ox = x.z; r[3].ox = x.w;
    r[0].oy = y.x; r[1].oy = y.y; r[2].oy = y.z; r[3].oy = y.w;
    r[0].oz = z.x; r[1].oz = z.y; r[2].oz = z.z; r[3].oz = z.w;
    if (kGather) {
        const float4 u = st[4 * n + i], v = st[5 * n + i], w = st[6 * n + i];
        r[0].vx = u.x; r[1].vx = u.y; r[2].vx = u.z; r[3].vx = u.w;
        r[0].vy = v.x; r[1].vy = v.y; r[2].vy = v.z; r[3].vy = v.w;
        r[0].vz = w.x; r[1].vz = w.y; r[2].vz = w.z; r[3].vz = w.w;
    } else {
#pragma unroll
        for (int j = 0; j < 4; ++j) r[j].vx = r[j].vy = r[j].vz = 0.f;
    }
}

// Record input: the push right after a cell sort reads the sort's 32-byte
// records (cell, offsets | velocities, id) instead of the word arrays, and
// writes the word arrays, so the sort needs no pass of its own to turn the
// records back into arrays.  A quad's eight 16-byte record halves are
// a0 b0 a1 b1 a2 b2 a3 b3 (a = cell and offsets, b = velocities and id); the
// first seven go through the stage slots the seven arrays use, and b3 is
// loaded into registers at the start of the quad's iteration.
//
// The warp stages its 32 quads together, as rows of the seven staged halves
// (112 bytes per quad, the warp's 3.5 KB where the arrays' seven slots per
// thread would be).  In copy k, lane l takes half t = l & 7 of quad
// 4k + (l >> 3), so a copy instruction reads one 512-byte span of records and
// its 28 active lanes write 448 contiguous bytes of the stage; lanes with t = 7
// (a b3 half) sit out.  A thread then reads its own row: rows of seven 16-byte
// slots put the eight lanes of a quarter-warp in eight different bank groups.
// Every lane of the warp runs this; quads at or past g1 are skipped.
__device__ __forceinline__ void prefetch_rec_warp(float4 *st, const int4 *rec, int64_t base, int64_t g1)
{
    const int lane = (int)(threadIdx.x & 31u), first = (int)(threadIdx.x & ~31u);
    const int t = lane & 7;
    const int64_t wq = base + first;          // the warp's first quad
    float4 *rows = st + 7 * first;
    if (t != 7) {
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int o = 4 * k + (lane >> 3);
            if (wq + o < g1) cp_async16(rows + 7 * o + t, rec + 8 * (wq + o) + t);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

// The thread's row was filled by other lanes of its warp: every lane waits for
// its own copies, then the warp barrier makes them visible across the warp.
__device__ __forceinline__ void read_rec(const float4 *st, const int4 &b3, P32 r[4], uint4 &id)
{
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncwarp();
    const float4 *row = st + 7 * threadIdx.x;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float4 a = row[2 * j];
        r[j].cell = __float_as_int(a.x);
        r[j].ox = a.y; r[j].oy = a.z; r[j].oz = a.w;
    }
    const float4 b0 = row[1], b1 = row[3], b2 = row[5];
    r[0].vx = b0.x; r[0].vy = b0.y; r[0].vz = b0.z;
    r[1].vx = b1.x; r[1].vy = b1.y; r[1].vz = b1.z;
    r[2].vx = b2.x; r[2].vy = b2.y; r[2].vz = b2.z;
    r[3].vx = __int_as_float(b3.x); r[3].vy = __int_as_float(b3.y); r[3].vz = __int_as_float(b3.z);
    id = make_uint4(__float_as_uint(b0.w), __float_as_uint(b1.w), __float_as_uint(b2.w), (unsigned)b3.w);
}

__device__ __forceinline__ void store_quad(const PartF32 &p, int64_t g, const P32 r[4])
{
    *(int4 *)(p.cell + 4 * g) = make_int4(r[0].cell, r[1].cell, r[2].cell, r[3].cell);
    *(float4 *)(p.ox + 4 * g) = make_float4(r[0].ox, r[1].ox, r[2].ox, r[3].ox);
    *(float4 *)(p.oy + 4 * g) = make_float4(r[0].oy, r[1].oy, r[2].oy, r[3].oy);
    *(float4 *)(p.oz + 4 * g) = make_float4(r[0].oz, r[1].oz, r[2].oz, r[3].oz);
    *(float4 *)(p.vx + 4 * g) = make_float4(r[0].vx, r[1].vx, r[2].vx, r[3].vx);
    *(float4 *)(p.vy + 4 * g) = make_float4(r[0].vy, r[1].vy, r[2].vy, r[3].vy);
    *(float4 *)(p.vz + 4 * g) = make_float4(r[0].vz, r[1].vz, r[2].vz, r[3].vz);
}

// FP32 Boris constants of one species.
struct Push32 {
    float hq;            // qm*dt/2: E -> half kick of the velocity
    float dt;
    float t0, t1, t2, s0, s1, s2;
};

// Per-thread diagnostics.
struct Tally {
    unsigned cx = 0, cy = 0, cz = 0, out = 0;
    float ke = 0.f, px = 0.f, py = 0.f, pz = 0.f;
};

// One particle's E at its 8 nodes, interpolated with component C of the pair
// weights ww: from the staged box when key >= 0, else from the padded global E
// (the particle left its box; nout counts it when `outside`).  The global node
// index is 32-bit whenever the padded grid has at most 2^32 nodes.
template <int C>
__device__ __forceinline__ float3 gather1(const TileArgs &a, const Box &box, int key, bool outside, int ix, int iy,
                                          int iz, const float4 *sE, const float2 ww[8], unsigned &nout)
{
    float4 nd[8];
    if (key >= 0) {
        const float4 *q = sE + key;
        nd[0] = q[0];
        nd[1] = q[1];
        nd[2] = q[box.sx];
        nd[3] = q[box.sx + 1];
        nd[4] = q[box.sxy];
        nd[5] = q[box.sxy + 1];
        nd[6] = q[box.sxy + box.sx];
        nd[7] = q[box.sxy + box.sx + 1];
    } else {
        nout += outside;
        const Geom &g = a.g;
        const float4 *E = (const float4 *)a.epad;
        const unsigned gx = (unsigned)g.gx, gxy = (unsigned)g.gx * (unsigned)g.gy;
        const float4 *q;
        if ((unsigned long long)gxy * (unsigned)g.gz <= 0xffffffffull)
            q = E + ((unsigned)(ix + g.halo) + gx * (unsigned)(iy + g.halo) + gxy * (unsigned)(iz + g.halo));
        else
            q = E + (ix + g.halo) + (int64_t)gx * (iy + g.halo) + (int64_t)gxy * (iz + g.halo);
        nd[0] = __ldg(q);
        nd[1] = __ldg(q + 1);
        nd[2] = __ldg(q + gx);
        nd[3] = __ldg(q + gx + 1);
        nd[4] = __ldg(q + gxy);
        nd[5] = __ldg(q + gxy + 1);
        nd[6] = __ldg(q + gxy + gx);
        nd[7] = __ldg(q + gxy + gx + 1);
    }
    float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll
    for (int n = 0; n < 8; ++n) {
        const float w = C == 0 ? ww[n].x : ww[n].y;
        ex = fmaf(nd[n].x, w, ex);
        ey = fmaf(nd[n].y, w, ey);
        ez = fmaf(nd[n].z, w, ez);
    }
    return make_float3(ex, ey, ez);
}

// Offset o in cell units after the move: the integer part goes to the cell
// index, o keeps the fraction in [0, 1).  o - floor(o) rounds to 1 for a
// negative o closer to 0 than half an ulp of 1; that particle keeps the lower
// cell at the largest offset below 1, a position within FP32 rounding of its
// true one like every other (one min instead of a test, a select and an add).
__device__ __forceinline__ void carry(float &o, float f, int &i)
{
    o = fminf(o, 0x1.fffffep-1f);
    i += (int)f;
}

// Two particles s0, s1 (v0, v1: slot inside the species' count): gather (MODE !=
// DEPOSIT), Boris + offset update + periodic cell wrap (PUSH/MOVE), interp output
// (INTERP) and the fixed-point CIC weights of the (new) position (PUSH/DEPOSIT).
// Each particle's arithmetic is the scalar sequence the reference writes
// (particle_mover_boris.f90:42-62, linear_interpolator.f90:54-66), carried for
// both particles by the pair instructions above.  dk[p] is the box index of
// particle p's deposit cell, or -1 when it has no shared deposit (no deposit
// mode, a slot past the count, or outside the box: then its weights already went
// to global memory).  A slot past the count is computed on a stand-in cell in
// the box and neither deposits, counts nor writes interp output.
template <int MODE, int W>
__device__ __forceinline__ void advance_pair(const TileArgs &a, const Box &box, bool e_ok, const float4 *sE, int sp,
                                             const Push32 &k, int64_t idx, bool v0, bool v1, P32 &s0, P32 &s1,
                                             unsigned u0[8], unsigned u1[8], int dk[2], Tally &t)
{
    constexpr bool kGather = MODE != MODE_DEPOSIT;
    constexpr bool kMove = MODE == MODE_PUSH || MODE == MODE_MOVE;
    constexpr bool kDeposit = MODE == MODE_PUSH || MODE == MODE_DEPOSIT;
    const Geom &g = a.g;
    // Cells are valid by construction: uploads and the injector wrap positions
    // into the grid (flagging anything else), the push wraps every cell it
    // writes, and a restored snapshot is checked on load.  So no per-particle
    // range check here (it cost 2.5% of the push).
    const int32_t standin = pack_cell(box.ox + g.halo, box.oy + g.halo, box.oz + g.halo);
    if (!v0) s0.cell = standin;
    if (!v1) s1.cell = standin;
    int ix0 = cell_x(s0.cell), iy0 = cell_y(s0.cell), iz0 = cell_z(s0.cell);
    int ix1 = cell_x(s1.cell), iy1 = cell_y(s1.cell), iz1 = cell_z(s1.cell);
    float2 ox = make_float2(s0.ox, s1.ox), oy = make_float2(s0.oy, s1.oy), oz = make_float2(s0.oz, s1.oz);
    if (kGather) {
        const int key0 = box.key(ix0, iy0, iz0), key1 = box.key(ix1, iy1, iz1);
        float2 wx0, wx1, wy0, wy1, wz0, wz1;
        cic2<W>(ox, wx0, wx1);
        cic2<W>(oy, wy0, wy1);
        cic2<W>(oz, wz0, wz1);
        const float2 a00 = mul2(wx0, wy0), a10 = mul2(wx1, wy0), a01 = mul2(wx0, wy1), a11 = mul2(wx1, wy1);
        const float2 ww[8] = {mul2(a00, wz0), mul2(a10, wz0), mul2(a01, wz0), mul2(a11, wz0),
                              mul2(a00, wz1), mul2(a10, wz1), mul2(a01, wz1), mul2(a11, wz1)};
        // (a slot past the count has the stand-in cell, inside the box)
        const float3 e0 = gather1<0>(a, box, e_ok ? key0 : -1, key0 < 0, ix0, iy0, iz0, sE, ww, t.out);
        const float3 e1 = gather1<1>(a, box, e_ok ? key1 : -1, key1 < 0, ix1, iy1, iz1, sE, ww, t.out);
        if (MODE == MODE_INTERP) {
            double *o = a.interp_out + 3 * idx;
            if (v0) { o[0] = e0.x; o[1] = e0.y; o[2] = e0.z; }
            if (v1) { o[3] = e1.x; o[4] = e1.y; o[5] = e1.z; }
        }
        if (kMove) {
            // Boris rotation with per-species t and s (particle_mover_boris.f90:42-56):
            // u- = v + h, u' = u- + u- x t, v = u- + u' x s + h with h = qm dt/2 E.
            // Each cross-product component b*c' - c*b' rounds the second product
            // first (multiplied by the negated constant: exact) and adds it in an FMA.
            const float2 hq = bc2(k.hq);
            const float2 hx = mul2(hq, make_float2(e0.x, e1.x));
            const float2 hy = mul2(hq, make_float2(e0.y, e1.y));
            const float2 hz = mul2(hq, make_float2(e0.z, e1.z));
            const float2 um0 = add2(make_float2(s0.vx, s1.vx), hx);
            const float2 um1 = add2(make_float2(s0.vy, s1.vy), hy);
            const float2 um2 = add2(make_float2(s0.vz, s1.vz), hz);
            const float2 ua0 = add2(um0, fma2(um1, bc2(k.t2), mul2(um2, bc2(-k.t1))));
            const float2 ua1 = add2(um1, fma2(um2, bc2(k.t0), mul2(um0, bc2(-k.t2))));
            const float2 ua2 = add2(um2, fma2(um0, bc2(k.t1), mul2(um1, bc2(-k.t0))));
            const float2 vx = add2(add2(um0, fma2(ua1, bc2(k.s2), mul2(ua2, bc2(-k.s1)))), hx);
            const float2 vy = add2(add2(um1, fma2(ua2, bc2(k.s0), mul2(ua0, bc2(-k.s2)))), hy);
            const float2 vz = add2(add2(um2, fma2(ua0, bc2(k.s1), mul2(ua1, bc2(-k.s0)))), hz);
            // Offset update in cell units (:60-62); a crossing moves the integer
            // cell and keeps the offset in [0, 1).
            ox = fma2(vx, bc2(k.dt), ox);
            oy = fma2(vy, bc2(k.dt), oy);
            oz = fma2(vz, bc2(k.dt), oz);
            const float2 fx = make_float2(floorf(ox.x), floorf(ox.y));
            const float2 fy = make_float2(floorf(oy.x), floorf(oy.y));
            const float2 fz = make_float2(floorf(oz.x), floorf(oz.y));
            ox = fma2(fx, bc2(-1.f), ox);
            oy = fma2(fy, bc2(-1.f), oy);
            oz = fma2(fz, bc2(-1.f), oz);
            carry(ox.x, fx.x, ix0); carry(ox.y, fx.y, ix1);
            carry(oy.x, fy.x, iy0); carry(oy.y, fy.y, iy1);
            carry(oz.x, fz.x, iz0); carry(oz.y, fz.y, iz1);
            // Periodic wrap of the cell (periodic_particle_boundary.f90:42-53); one
            // branch for both particles and all axes, taken only at the box faces.
            const bool out0 = (unsigned)ix0 >= (unsigned)g.nx || (unsigned)iy0 >= (unsigned)g.ny ||
                              (unsigned)iz0 >= (unsigned)g.nz;
            const bool out1 = (unsigned)ix1 >= (unsigned)g.nx || (unsigned)iy1 >= (unsigned)g.ny ||
                              (unsigned)iz1 >= (unsigned)g.nz;
            if (out0 || out1) {
                if (v0) {
                    t.cx += (unsigned)ix0 >= (unsigned)g.nx;
                    t.cy += (unsigned)iy0 >= (unsigned)g.ny;
                    t.cz += (unsigned)iz0 >= (unsigned)g.nz;
                }
                if (v1) {
                    t.cx += (unsigned)ix1 >= (unsigned)g.nx;
                    t.cy += (unsigned)iy1 >= (unsigned)g.ny;
                    t.cz += (unsigned)iz1 >= (unsigned)g.nz;
                }
                ix0 = wrapi(ix0, g.nx); iy0 = wrapi(iy0, g.ny); iz0 = wrapi(iz0, g.nz);
                ix1 = wrapi(ix1, g.nx); iy1 = wrapi(iy1, g.ny); iz1 = wrapi(iz1, g.nz);
            }
            s0.ox = ox.x; s0.oy = oy.x; s0.oz = oz.x;
            s1.ox = ox.y; s1.oy = oy.y; s1.oz = oz.y;
            s0.vx = vx.x; s0.vy = vy.x; s0.vz = vz.x;
            s1.vx = vx.y; s1.vy = vy.y; s1.vz = vz.y;
            s0.cell = pack_cell(ix0, iy0, iz0);
            s1.cell = pack_cell(ix1, iy1, iz1);
            if (a.with_energy) {
                if (v0) {
                    t.ke = fmaf(vx.x, vx.x, fmaf(vy.x, vy.x, fmaf(vz.x, vz.x, t.ke)));
                    t.px += vx.x; t.py += vy.x; t.pz += vz.x;
                }
                if (v1) {
                    t.ke = fmaf(vx.y, vx.y, fmaf(vy.y, vy.y, fmaf(vz.y, vz.y, t.ke)));
                    t.px += vx.y; t.py += vy.y; t.pz += vz.y;
                }
            }
        }
    }
    dk[0] = dk[1] = -1;
    if (!kDeposit) return;
    fixed_weights2<W>(ox, oy, oz, u0, u1);
    const int d0 = box.key(ix0, iy0, iz0), d1 = box.key(ix1, iy1, iz1);
    const bool g0 = v0 && d0 < 0, g1 = v1 && d1 < 0;
    if (g0 || g1) {
        unsigned long long *w = a.wsum + (int64_t)sp * g.ncell;
        if (g0) deposit_global_fixed(g, w, ix0, iy0, iz0, u0);
        if (g1) deposit_global_fixed(g, w, ix1, iy1, iz1, u1);
        if (!kGather) t.out += (unsigned)g0 + (unsigned)g1;
    }
    if (v0) dk[0] = d0;
    if (v1) dk[1] = d1;
}

// A thread whose bounded wait for the E box gave up has gathered from global
// memory, but the copy may still be landing in this CTA's shared memory.  It
// waits the copy out (bounded again) before the CTA can finish and release that
// memory; a copy that never completes leaves a second error site.
__device__ __forceinline__ void drain_tma(const TileArgs &a, bool lost, uint64_t *ebar)
{
    if (lost && !mbar_wait(ebar, 0, kTmaWaitPolls)) flag_error(a.diag, OHPIC_ERR_TIMEOUT, 7);
}

// Two consecutive particles per lane (8-byte vector loads and stores); the
// pair's weights are summed in registers when both fall in one cell, then the
// warp combines lanes sharing a cell (warp_run_deposit), a second round only
// for pairs that split.  The next pair is loaded before the current one is
// computed.
//
// One work item (a tile's particle range of one species) of one context.  smem
// is the dynamic shared memory (E box, then the deposit box), ebar an mbarrier
// for the TMA copy of the E box; emap may be null when a.use_tma is 0.
template <int MODE, int DEP, int W>
__device__ __forceinline__ void tile_pass(const TileArgs &a, const PartF32 &p, const CUtensorMap *emap,
                                          const Item &it, unsigned char *smem, uint64_t *ebar)
{
    constexpr bool kGather = MODE != MODE_DEPOSIT;
    constexpr bool kMove = MODE == MODE_PUSH || MODE == MODE_MOVE;
    constexpr bool kDeposit = MODE == MODE_PUSH || MODE == MODE_DEPOSIT;

    const Geom &g = a.g;
    const Box box = make_box(g, it);
    const int s3 = g.sx * g.sy * g.sz;
    float4 *sE = (float4 *)smem;
    unsigned *slo = (unsigned *)(smem + (kGather ? (size_t)s3 * sizeof(float4) : 0));
    unsigned *shi = slo + s3;
    // The E box arrives by one TMA copy while the threads clear the deposit box.
    const bool tma = box.on && kGather && a.use_tma && emap != nullptr;
    if (tma && threadIdx.x == 0) {
        mbar_init(ebar, 1);
        mbar_expect_tx(ebar, (uint32_t)(s3 * sizeof(float4)));
        tma_load_3d(sE, emap, 4 * it.x0, it.y0, it.z0, ebar);
    }
    if (box.on) {
        stage_f32(a, it, sE, slo, shi, kGather && !tma, kDeposit);
        __syncthreads();
    }
    bool e_ok = box.on;
    const bool lost = tma && !mbar_wait(ebar, 0, a.tma_polls);
    if (lost) {
        flag_error(a.diag, OHPIC_ERR_TIMEOUT, 5);
        e_ok = false;   // gather from global memory instead
    }

    const int sp = it.sp;
    const SpeciesConst &c = a.sc[sp];
    Push32 k;
    k.hq = c.hq32;
    k.dt = c.dt32;
    k.t0 = c.t32[0]; k.t1 = c.t32[1]; k.t2 = c.t32[2];
    k.s0 = c.s32[0]; k.s1 = c.s32[1]; k.s2 = c.s32[2];
    const int64_t end = a.seg[sp] + a.count[sp];
    Tally t;

    int64_t gi = it.g0 + threadIdx.x;
    bool gv = gi < it.g1;
    P32 cur[2];
    if (gv) load_pair<kGather>(p, gi, cur);
    for (int64_t base = it.g0; base < it.g1; base += blockDim.x) {
        const int64_t gn = gi + blockDim.x;
        const bool vn = gn < it.g1;
        P32 nxt[2];
        if (vn) load_pair<kGather>(p, gn, nxt);

        int k0 = -1, k1 = -1;
        unsigned u0[8], u1[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) u0[v] = u1[v] = 0u;
        if (gv) {
            int dk[2];
            advance_pair<MODE, W>(a, box, e_ok, sE, sp, k, 2 * gi, 2 * gi < end, 2 * gi + 1 < end, cur[0], cur[1],
                                  u0, u1, dk, t);
            k0 = dk[0];
            k1 = dk[1];
            if (kMove) store_pair(p, gi, cur);
        }
        if (kDeposit) {
            if (k0 >= 0 && k1 == k0) {
#pragma unroll
                for (int v = 0; v < 8; ++v) u0[v] += u1[v];
                k1 = -1;
            }
            warp_run_deposit<DEP>(k0, u0, slo, shi, box.sx, box.sxy);
            if (__any_sync(kFull, k1 >= 0)) warp_run_deposit<DEP>(k1, u1, slo, shi, box.sx, box.sxy);
        }
        gi = gn;
        gv = vn;
        cur[0] = nxt[0];
        cur[1] = nxt[1];
    }
    drain_tma(a, lost, ebar);
    if (kDeposit && box.on) {
        __syncthreads();
        flush_f32(a, it, slo, shi);
    }
    if (kMove || kGather) flush_diag<float>(a, sp, t.cx, t.cy, t.cz, t.out, t.ke, t.px, t.py, t.pz);
}

// The same work item with four consecutive particles per lane (16-byte vectors,
// PUSH and DEPOSIT only).  A lane's particles are cell-sorted neighbours, so it
// sums their fixed-point weights in registers while the cell stays the same,
// adds to the shared box directly when its cell changes, and the warp combines
// the lanes' last sums once per 128 particles.  The per-particle arithmetic is
// advance_pair(), as in the two-per-lane pass, and every sum is integer, so both
// passes give the same bits.
template <int MODE, int DEP, int W, bool REC = false, bool FIX = false>
__device__ __forceinline__ void tile_pass4(const TileArgs &a, const PartF32 &p, const CUtensorMap *emap,
                                           const Item &it, unsigned char *smem, uint64_t *ebar,
                                           const RecIn &rin = RecIn{})
{
    static_assert(MODE == MODE_PUSH || MODE == MODE_DEPOSIT, "four per lane: push or deposit");
    static_assert(!REC || MODE == MODE_PUSH, "record input: push only");
    constexpr bool kGather = MODE != MODE_DEPOSIT;
    constexpr bool kMove = MODE == MODE_PUSH;

    const Geom &g = a.g;
    Box box = make_box(g, it);
    if constexpr (FIX) {
        // the box of tile (16,8,8) with halo 2, its spans and pitches immediates
        box.spx = kFixTx + 2 * kFixHalo;
        box.spy = kFixTy + 2 * kFixHalo;
        box.spz = kFixTz + 2 * kFixHalo;
        box.sx = kFixTx + 2 * kFixHalo + 1;
        box.sxy = box.sx * (kFixTy + 2 * kFixHalo + 1);
    }
    const int s3 = FIX ? box.sxy * (kFixTz + 2 * kFixHalo + 1) : g.sx * g.sy * g.sz;
    float4 *sE = (float4 *)smem;
    unsigned *slo = (unsigned *)(smem + (kGather ? (size_t)s3 * sizeof(float4) : 0));
    unsigned *shi = slo + s3;
    const bool tma = box.on && kGather && a.use_tma && emap != nullptr;
    if (tma && threadIdx.x == 0) {
        mbar_init(ebar, 1);
        mbar_expect_tx(ebar, (uint32_t)(s3 * sizeof(float4)));
        tma_load_3d(sE, emap, 4 * it.x0, it.y0, it.z0, ebar);
    }
    if (box.on) {
        stage_f32(a, it, sE, slo, shi, kGather && !tma, true);
        __syncthreads();
    }
    bool e_ok = box.on;
    const bool lost = tma && !mbar_wait(ebar, 0, a.tma_polls);
    if (lost) {
        flag_error(a.diag, OHPIC_ERR_TIMEOUT, 6);
        e_ok = false;
    }

    const int sp = it.sp;
    const SpeciesConst &c = a.sc[sp];
    Push32 k;
    k.hq = c.hq32;
    k.dt = c.dt32;
    k.t0 = c.t32[0]; k.t1 = c.t32[1]; k.t2 = c.t32[2];
    k.s0 = c.s32[0]; k.s1 = c.s32[1]; k.s2 = c.s32[2];
    const int64_t end = a.seg[sp] + a.count[sp];
    Tally t;
    // Prefetch stage after the boxes (16-byte aligned); the launch reserves it.
    const size_t boxes = box.on ? ((kGather ? (size_t)s3 * sizeof(float4) : 0) + (size_t)s3 * 8 + 15) & ~(size_t)15 : 0;
    float4 *stage = (float4 *)(smem + boxes);
    if (REC) {
        prefetch_rec_warp(stage, rin.rec, it.g0, it.g1);
    } else if (it.g0 + threadIdx.x < it.g1) {
        prefetch_quad<kGather>(stage, p, it.g0 + threadIdx.x);
    }

    for (int64_t base = it.g0; base < it.g1; base += blockDim.x) {
        const int64_t gi = base + threadIdx.x;
        int acc_key = -1;
        unsigned acc[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) acc[v] = 0u;
        P32 q[4];
        if (REC) {
            // The quad's last record half, loaded here and first used by the
            // second pair: its 32-byte sector came into L2 with the staged copy of
            // the same quad's a3 half, one iteration ago.
            const int4 b3 = gi < it.g1 ? __ldg(rin.rec + 8 * gi + 7) : make_int4(0, 0, 0, 0);
            uint4 qid;
            // the whole warp: its lanes read each other's copies, and the next
            // copies overwrite the stage only after every lane has read it
            read_rec(stage, b3, q, qid);
            __syncwarp();
            if (base + blockDim.x < it.g1) prefetch_rec_warp(stage, rin.rec, base + blockDim.x, it.g1);
            // the ids go out at once, so they hold no registers through the quad
            if (rin.ids && gi < it.g1) *(uint4 *)(rin.ids + 4 * gi) = qid;
        }
        if (gi < it.g1) {
            if (!REC) {
                read_quad<kGather>(stage, q);
                if (gi + blockDim.x < it.g1) prefetch_quad<kGather>(stage, p, gi + blockDim.x);
            }
            // particles of the quad inside the species' count (4 but at its end)
            const int nv = (int)min(end - 4 * gi, (int64_t)4);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int64_t i0 = 4 * gi + 2 * h;
                unsigned ua[8], ub[8];
                int dk[2];
                advance_pair<MODE, W>(a, box, e_ok, sE, sp, k, i0, 2 * h < nv, 2 * h + 1 < nv, q[2 * h],
                                      q[2 * h + 1], ua, ub, dk, t);
                // A run ends where the key changes; a particle with no shared
                // deposit (key -1) ends it too and starts an empty one.
#pragma unroll
                for (int p2 = 0; p2 < 2; ++p2) {
                    const unsigned *u = p2 ? ub : ua;
                    if (dk[p2] != acc_key) {
                        if (acc_key >= 0) box_add8(shi, slo, acc_key, box.sx, box.sxy, acc);
                        acc_key = dk[p2];
#pragma unroll
                        for (int v = 0; v < 8; ++v) acc[v] = u[v];
                    } else {
#pragma unroll
                        for (int v = 0; v < 8; ++v) acc[v] += u[v];
                    }
                }
            }
            if (kMove) store_quad(p, gi, q);
        }
        warp_run_deposit<DEP>(acc_key, acc, slo, shi, box.sx, box.sxy);
    }
    drain_tma(a, lost, ebar);
    if (box.on) {
        __syncthreads();
        flush_f32(a, it, slo, shi);
    }
    if (kGather) flush_diag<float>(a, sp, t.cx, t.cy, t.cz, t.out, t.ke, t.px, t.py, t.pz);
}

// The dynamic shared memory from its first 128-byte boundary (the launch
// reserves the slack).  The offset is added to the shared array itself: a
// round trip of the pointer through an integer hides its address space, and the
// box loads and atomics then compile to generic instructions (18 loads and 8
// atomics per particle in the push) instead of shared-memory ones.
__device__ __forceinline__ unsigned char *align128(unsigned char *p)
{
    return p + ((128u - (smem_addr(p) & 127u)) & 127u);
}

// Work item b with PPL particles per lane: 2 (every mode) or 4 (push and deposit).
template <int MODE, int DEP, int PPL, int W, bool FIX = false>
__device__ __forceinline__ void run_item(const TileArgs &a, const PartF32 &p, const CUtensorMap *emap, int64_t b,
                                         unsigned char *smem, uint64_t *ebar)
{
    Item it;
    if constexpr (PPL == 4) {
        if (get_item<4>(a, b, it)) tile_pass4<MODE, DEP, W, false, FIX>(a, p, emap, it, smem, ebar);
    } else {
        if (get_item<2>(a, b, it)) tile_pass<MODE, DEP, W>(a, p, emap, it, smem, ebar);
    }
}

// One context: one CTA per work item.  FIX: the launch's tile is (16,8,8) with
// halo 2, so the box spans and pitches are compile-time constants.
template <int MODE, int DEP, int PPL, int W, bool FIX = false>
__global__ void __launch_bounds__(256, 2) tiled_f32(TileArgs a, PartF32 p, const __grid_constant__ CUtensorMap emap)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t ebar;
    // box start aligned to 128 bytes (the launch reserves the slack)
    run_item<MODE, DEP, PPL, W, FIX>(a, p, &emap, (int64_t)blockIdx.x, align128(smem_raw), &ebar);
}

// The push right after a sort, reading the sort's records (four per lane, LANES
// deposit: the default launch shape); writes the word arrays p and the ids.
template <int W, bool FIX>
__global__ void __launch_bounds__(256, 2) tiled_f32_rec(TileArgs a, PartF32 p, RecIn rin,
                                                        const __grid_constant__ CUtensorMap emap)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t ebar;
    Item it;
    if (get_item<4>(a, (int64_t)blockIdx.x, it))
        tile_pass4<MODE_PUSH, OHPIC_DEPOSIT_LANES, W, true, FIX>(a, p, &emap, it, align128(smem_raw), &ebar, rin);
}

// Many contexts in one persistent launch.  Every CTA takes the next item from
// one queue over all runs (an atomic cursor), looks up its run in the
// inclusive item prefix held in shared memory, copies that run's descriptor to
// shared memory when the run changes, and runs the same tile pass.  Runs are
// ordered by decreasing particles per item, so the queue hands out the long
// items first.
template <int MODE, int DEP, int PPL, int W>
__global__ void __launch_bounds__(256, 2) tiled_f32_multi(MultiPush m)
{
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(16) RunDesc sd;
    __shared__ int64_t s_end[kMaxServeRuns];
    __shared__ int64_t s_item;
    __shared__ int s_run;
    __shared__ __align__(8) uint64_t ebar;
    const int nruns = *m.nruns;
    for (int i = threadIdx.x; i < nruns; i += blockDim.x) s_end[i] = m.item_end[i];
    __syncthreads();
    const int64_t total = nruns > 0 ? s_end[nruns - 1] : 0;
    unsigned char *smem = align128(smem_raw);
    int cur = -1;
    for (;;) {
        if (threadIdx.x == 0) {
            const int64_t item = (int64_t)atomicAdd(m.cursor, 1ull);
            int lo = 0, hi = nruns - 1;
            while (lo < hi) {   // first run whose inclusive end exceeds item
                const int mid = (lo + hi) >> 1;
                if (s_end[mid] > item) hi = mid;
                else lo = mid + 1;
            }
            s_item = item;
            s_run = lo;
        }
        __syncthreads();
        const int64_t item = s_item;
        const int r = s_run;
        if (item >= total) break;
        if (r != cur) {
            const unsigned *src = (const unsigned *)(m.runs + r);
            unsigned *dst = (unsigned *)&sd;
            for (int i = threadIdx.x; i < (int)(sizeof(RunDesc) / 4); i += blockDim.x) dst[i] = src[i];
            cur = r;
            __syncthreads();
        }
        // The descriptor is read in place from shared memory.  A private copy
        // (about 1 KB per thread, its per-species arrays indexed at run time)
        // lands in local memory and costs 256 KB of local stores per item.
        const TileArgs &a = sd.a;
        const PartF32 &p = sd.p;
        run_item<MODE, DEP, PPL, W>(a, p, nullptr, item - (r > 0 ? s_end[r - 1] : 0), smem, &ebar);
        __syncthreads();   // the next item reuses the shared boxes and descriptor
    }
}

}  // namespace

template <typename P>
static void launch_k(ohpic_ctx *c, void (*kernel)(TileArgs, P, const CUtensorMap), const TileArgs &a,
                     int64_t blocks, size_t smem, const P &parts)
{
    if (blocks <= 0) return;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // CTAs over ~96 KB pair up on an SM only with the whole shared-memory carveout
    if (smem > 96 * 1024)
        cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    kernel<<<(unsigned)blocks, 256, smem, c->stream>>>(a, parts, c->emap);
    ++c->launches;
}

// The deposit strategy and the particles per lane are template parameters;
// these map the run-time choices.
template <typename F>
static auto by_deposit(int dep, F f)
{
    switch (dep) {
    case OHPIC_DEPOSIT_MATCH: return f(std::integral_constant<int, OHPIC_DEPOSIT_MATCH>());
    case OHPIC_DEPOSIT_UNIFORM: return f(std::integral_constant<int, OHPIC_DEPOSIT_UNIFORM>());
    case OHPIC_DEPOSIT_GROUPS: return f(std::integral_constant<int, OHPIC_DEPOSIT_GROUPS>());
    case OHPIC_DEPOSIT_LANES: return f(std::integral_constant<int, OHPIC_DEPOSIT_LANES>());
    default: return f(std::integral_constant<int, OHPIC_DEPOSIT_RUNS>());
    }
}

template <typename F>
static auto by_lanes(int ppl, F f)
{
    if (ppl == 4) return f(std::integral_constant<int, 4>());
    return f(std::integral_constant<int, 2>());
}

template <typename F>
static auto by_weights(int w, F f)
{
    if (w == OHPIC_WEIGHTS_REFERENCE) return f(std::integral_constant<int, OHPIC_WEIGHTS_REFERENCE>());
    return f(std::integral_constant<int, OHPIC_WEIGHTS_STANDARD>());
}

void launch_tiled_f32(ohpic_ctx *c, const TileArgs &a, int mode, int64_t blocks, size_t smem, const RecIn *rin)
{
    const PartF32 &pp = c->p32[c->cur];
    const Geom &g = a.g;
    const bool fix = g.tx == kFixTx && g.ty == kFixTy && g.tz == kFixTz && g.halo == kFixHalo;
    by_weights(a.weights, [&](auto w) {
        constexpr int W = decltype(w)::value;
        if (rin) {
            if (blocks <= 0) return 0;
            auto kernel = fix ? tiled_f32_rec<W, true> : tiled_f32_rec<W, false>;
            cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (smem > 96 * 1024)
                cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared);
            kernel<<<(unsigned)blocks, 256, smem, c->stream>>>(a, pp, *rin, c->emap);
            ++c->launches;
            return 0;
        }
        if (mode == MODE_PUSH || mode == MODE_DEPOSIT) {
            by_lanes(a.ppl, [&](auto l) {
                return by_deposit(a.deposit, [&](auto d) {
                    constexpr int D = decltype(d)::value, L = decltype(l)::value;
                    if (mode == MODE_PUSH && L == 4 && D == OHPIC_DEPOSIT_LANES && fix)
                        launch_k(c, tiled_f32<MODE_PUSH, D, L, W, true>, a, blocks, smem, pp);
                    else if (mode == MODE_PUSH) launch_k(c, tiled_f32<MODE_PUSH, D, L, W>, a, blocks, smem, pp);
                    else launch_k(c, tiled_f32<MODE_DEPOSIT, D, L, W>, a, blocks, smem, pp);
                    return 0;
                });
            });
        } else if (mode == MODE_MOVE) {
            launch_k(c, tiled_f32<MODE_MOVE, OHPIC_DEPOSIT_RUNS, 2, W>, a, blocks, smem, pp);
        } else {
            launch_k(c, tiled_f32<MODE_INTERP, OHPIC_DEPOSIT_RUNS, 2, W>, a, blocks, smem, pp);
        }
        return 0;
    });
}

template <int MODE, int DEP, int PPL, int W>
static cudaError_t launch_multi_k(cudaStream_t st, const MultiPush &m, int grid, size_t smem)
{
    auto kernel = tiled_f32_multi<MODE, DEP, PPL, W>;
    cudaError_t e = cudaSuccess;
    if (smem > 48 * 1024) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kernel<<<(unsigned)grid, 256, smem, st>>>(m);
    return cudaGetLastError();
}

cudaError_t launch_multi_f32(cudaStream_t st, int mode, int dep, int ppl, int weights, const MultiPush &m,
                             int grid, size_t smem)
{
    if (grid <= 0) return cudaSuccess;
    return by_weights(weights, [&](auto w) {
        return by_lanes(ppl, [&](auto l) {
            return by_deposit(dep, [&](auto d) {
                constexpr int D = decltype(d)::value, L = decltype(l)::value, W = decltype(w)::value;
                if (mode == MODE_DEPOSIT) return launch_multi_k<MODE_DEPOSIT, D, L, W>(st, m, grid, smem);
                return launch_multi_k<MODE_PUSH, D, L, W>(st, m, grid, smem);
            });
        });
    });
}

}  // namespace ohpic
