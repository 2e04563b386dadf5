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
// Mapping.  Lane l of a warp handles particle base + l, so the 32 lanes hold 32
// consecutive particles of the cell-sorted order: their cells are mostly the
// same one or two, the 8 node loads of the gather are shared-memory broadcasts,
// and their deposits form runs of equal cells across adjacent lanes.  Loads and
// stores are 4-byte coalesced accesses; the next batch's 7 values are loaded
// before the current batch is computed.
//
// Deposit in fixed point.  Each particle's 8 CIC weights are rounded to units of
// 2^-24 with the largest one adjusted so they sum to exactly 2^24 (charge is
// conserved exactly).  A warp segmented reduction (integer shuffles, at most 5
// steps, stopping early when runs are short) sums each run into its first lane,
// which adds the sums to a shared 64-bit box kept as 32-bit low/high words:
// 32-bit shared atomic adds are native and same-address adds within a warp do not
// serialise, unlike FP32 shared atomics.  The box is flushed once per CTA into
// per-species 64-bit global sums.  All of it is integer addition, so the deposit
// does not depend on the order in which atomics land.
#include "tile_common.cuh"
#include "tma.cuh"

namespace ohpic {
namespace {

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
#pragma unroll
    for (int v = 0; v < 8; ++v)
        if (old[v] + u[v] < old[v]) atomicAdd(hi + key + off[v], 1u);
}

// Adds u (weights, key = box index of the cell or < 0) to the shared box after
// combining the lanes that share a key.  DEP picks the combination
// (OHPIC_DEPOSIT_*): runs of adjacent lanes by shuffles; one hardware warp
// reduce when every lane holds the same key, else runs; or __match_any_sync
// groups reduced with __reduce_add_sync.  All 32 lanes must call this.
template <int DEP>
__device__ __forceinline__ void warp_run_deposit(int key, unsigned u[8], unsigned *lo, unsigned *hi, int sx,
                                                 int sxy)
{
    const unsigned lane = threadIdx.x & 31u;
    bool head;
    if (DEP == OHPIC_DEPOSIT_MATCH) {
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

// CIC weights of one particle in units of 2^-24, summing to exactly 2^24: the
// largest corner (the product of the larger weight on each axis, >= 1/8) takes
// the rounding remainder.
__device__ __forceinline__ void fixed_weights(int conv, float ox, float oy, float oz, unsigned u[8])
{
    float wx0, wx1, wy0, wy1, wz0, wz1;
    cic<float>(conv, ox, wx0, wx1);
    cic<float>(conv, oy, wy0, wy1);
    cic<float>(conv, oz, wz0, wz1);
    const float a00 = wx0 * wy0, a10 = wx1 * wy0, a01 = wx0 * wy1, a11 = wx1 * wy1;
    const float sz0 = wz0 * kWeightScale, sz1 = wz1 * kWeightScale;   // exact: power-of-two scale
    const float f[8] = {a00 * sz0, a10 * sz0, a01 * sz0, a11 * sz0, a00 * sz1, a10 * sz1, a01 * sz1, a11 * sz1};
    unsigned sum = 0;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
        u[v] = __float2uint_rn(f[v]);
        sum += u[v];
    }
    const int big = (wx1 > wx0 ? 1 : 0) + (wy1 > wy0 ? 2 : 0) + (wz1 > wz0 ? 4 : 0);
    const unsigned fix = (1u << 24) - sum;   // small, possibly "negative" (mod 2^32)
#pragma unroll
    for (int v = 0; v < 8; ++v) u[v] += v == big ? fix : 0u;
}

__device__ __forceinline__ void deposit_global_fixed(const Geom &g, unsigned long long *w, int ix, int iy, int iz,
                                                     const unsigned u[8])
{
    const int ix1 = ix + 1 == g.nx ? 0 : ix + 1;
    const int iy1 = iy + 1 == g.ny ? 0 : iy + 1;
    const int iz1 = iz + 1 == g.nz ? 0 : iz + 1;
    const int64_t y0 = (int64_t)iy * g.nx, y1 = (int64_t)iy1 * g.nx;
    const int64_t z0 = (int64_t)iz * g.nx * g.ny, z1 = (int64_t)iz1 * g.nx * g.ny;
    atomicAdd(w + ix + y0 + z0, (unsigned long long)u[0]);
    atomicAdd(w + ix1 + y0 + z0, (unsigned long long)u[1]);
    atomicAdd(w + ix + y1 + z0, (unsigned long long)u[2]);
    atomicAdd(w + ix1 + y1 + z0, (unsigned long long)u[3]);
    atomicAdd(w + ix + y0 + z1, (unsigned long long)u[4]);
    atomicAdd(w + ix1 + y0 + z1, (unsigned long long)u[5]);
    atomicAdd(w + ix + y1 + z1, (unsigned long long)u[6]);
    atomicAdd(w + ix1 + y1 + z1, (unsigned long long)u[7]);
}

// Shared box: E nodes (float4) then the low and high words of the weight sums.
__device__ __forceinline__ void stage_f32(const TileArgs &a, const Item &it, float4 *sE, unsigned *lo, unsigned *hi,
                                          bool need_e, bool need_w)
{
    // One box row (fixed y, z) per warp iteration, lanes along x.
    const Geom &g = a.g;
    const float4 *E = (const float4 *)a.epad;
    const int rows = g.sy * g.sz, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = threadIdx.x >> 5; r < rows; r += nw) {
        const int cz = r / g.sy, by = r - cz * g.sy;
        // padded index of node x0 - halo + ax is x0 + ax
        const float4 *src = E + ((int64_t)(it.z0 + cz) * g.gy + (it.y0 + by)) * g.gx + it.x0;
        const int base = r * g.sx;
        for (int ax = lane; ax < g.sx; ax += 32) {
            if (need_e) sE[base + ax] = __ldg(src + ax);
            if (need_w) {
                lo[base + ax] = 0u;
                hi[base + ax] = 0u;
            }
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

template <bool kGather>
__device__ __forceinline__ void load_p(const PartF32 &p, int64_t i, P32 &r)
{
    r.cell = p.cell[i];
    r.ox = p.ox[i];
    r.oy = p.oy[i];
    r.oz = p.oz[i];
    if (kGather) {
        r.vx = p.vx[i];
        r.vy = p.vy[i];
        r.vz = p.vz[i];
    } else {
        r.vx = r.vy = r.vz = 0.f;
    }
}

template <int MODE, int DEP>
__global__ void __launch_bounds__(256, 3) tiled_f32(TileArgs a, PartF32 p, const __grid_constant__ CUtensorMap emap)
{
    constexpr bool kGather = MODE != MODE_DEPOSIT;
    constexpr bool kMove = MODE == MODE_PUSH || MODE == MODE_MOVE;
    constexpr bool kDeposit = MODE == MODE_PUSH || MODE == MODE_DEPOSIT;

    Item it;
    if (!get_item<1>(a, it)) return;
    const Geom &g = a.g;
    const Box box = make_box(g, it);
    extern __shared__ unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t ebar;
    // box start aligned to 128 bytes (the launch reserves the slack)
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
    const int s3 = g.sx * g.sy * g.sz;
    float4 *sE = (float4 *)smem;
    unsigned *slo = (unsigned *)(smem + (kGather ? (size_t)s3 * sizeof(float4) : 0));
    unsigned *shi = slo + s3;
    // The E box arrives by one TMA copy while the threads clear the deposit box.
    const bool tma = box.on && kGather && a.use_tma;
    if (tma && threadIdx.x == 0) {
        mbar_init(&ebar, 1);
        mbar_expect_tx(&ebar, (uint32_t)(s3 * sizeof(float4)));
        tma_load_3d(sE, &emap, 4 * it.x0, it.y0, it.z0, &ebar);
    }
    if (box.on) {
        stage_f32(a, it, sE, slo, shi, kGather && !tma, kDeposit);
        __syncthreads();
    }
    bool e_ok = box.on;
    if (tma && !mbar_wait(&ebar, 0, kTmaWaitPolls)) {
        flag_error(a.diag, OHPIC_ERR_TIMEOUT, 5);
        e_ok = false;   // gather from global memory instead
    }

    const int sp = it.sp;
    const SpeciesConst &c = a.sc[sp];
    const float hq = (float)(c.qm * c.dt2);      // E -> half kick of the velocity
    const float dtf = (float)c.dt;
    const float t0 = (float)c.t[0], t1 = (float)c.t[1], t2 = (float)c.t[2];
    const float s0 = (float)c.s[0], s1 = (float)c.s[1], s2 = (float)c.s[2];
    unsigned ncx = 0, ncy = 0, ncz = 0, nout = 0;
    float ke = 0.f, px = 0.f, py = 0.f, pz = 0.f;

    int64_t i = it.g0 + threadIdx.x;
    bool valid = i < it.g1;
    P32 cur;
    if (valid) load_p<kGather>(p, i, cur);
    for (int64_t base = it.g0; base < it.g1; base += blockDim.x) {
        const int64_t inext = i + blockDim.x;
        const bool vnext = inext < it.g1;
        P32 nxt;
        if (vnext) load_p<kGather>(p, inext, nxt);

        int dkey = -1;
        unsigned w[8];
#pragma unroll
        for (int v = 0; v < 8; ++v) w[v] = 0u;
        if (valid) {
            int ix = cell_x(cur.cell), iy = cell_y(cur.cell), iz = cell_z(cur.cell);
            bool ok = ix < g.nx && iy < g.ny && iz < g.nz;
            if (!ok) flag_error(a.diag, OHPIC_ERR_BOUNDS, 3);
            if (ok && kGather) {
                const int key = box.key(ix, iy, iz);
                nout += key < 0;
                float wx0, wx1, wy0, wy1, wz0, wz1;
                cic<float>(a.weights, cur.ox, wx0, wx1);
                cic<float>(a.weights, cur.oy, wy0, wy1);
                cic<float>(a.weights, cur.oz, wz0, wz1);
                const float a00 = wx0 * wy0, a10 = wx1 * wy0, a01 = wx0 * wy1, a11 = wx1 * wy1;
                const float ww[8] = {a00 * wz0, a10 * wz0, a01 * wz0, a11 * wz0,
                                     a00 * wz1, a10 * wz1, a01 * wz1, a11 * wz1};
                float4 nd[8];
                load_nodes<float4>(a, box, e_ok ? key : -1, ix, iy, iz, sE, nd);
                float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll
                for (int n = 0; n < 8; ++n) {
                    ex = fmaf(nd[n].x, ww[n], ex);
                    ey = fmaf(nd[n].y, ww[n], ey);
                    ez = fmaf(nd[n].z, ww[n], ez);
                }
                if (MODE == MODE_INTERP) {
                    double *o = a.interp_out + 3 * i;
                    o[0] = ex;
                    o[1] = ey;
                    o[2] = ez;
                }
                if (kMove) {
                    // Boris rotation with per-species t and s (particle_mover_boris.f90:42-56).
                    const float hx = hq * ex, hy = hq * ey, hz = hq * ez;
                    const float um0 = cur.vx + hx, um1 = cur.vy + hy, um2 = cur.vz + hz;
                    const float ua0 = um0 + (um1 * t2 - um2 * t1);
                    const float ua1 = um1 + (um2 * t0 - um0 * t2);
                    const float ua2 = um2 + (um0 * t1 - um1 * t0);
                    cur.vx = um0 + (ua1 * s2 - ua2 * s1) + hx;
                    cur.vy = um1 + (ua2 * s0 - ua0 * s2) + hy;
                    cur.vz = um2 + (ua0 * s1 - ua1 * s0) + hz;
                    // Offset update in cell units; a crossing moves the integer cell
                    // (wrapped periodically) and keeps the offset in [0, 1).
                    float nxo = fmaf(cur.vx, dtf, cur.ox);
                    float nyo = fmaf(cur.vy, dtf, cur.oy);
                    float nzo = fmaf(cur.vz, dtf, cur.oz);
                    float fx = floorf(nxo), fy = floorf(nyo), fz = floorf(nzo);
                    nxo -= fx; nyo -= fy; nzo -= fz;
                    if (nxo >= 1.f) { nxo = 0.f; fx += 1.f; }
                    if (nyo >= 1.f) { nyo = 0.f; fy += 1.f; }
                    if (nzo >= 1.f) { nzo = 0.f; fz += 1.f; }
                    ix += (int)fx; iy += (int)fy; iz += (int)fz;
                    if ((unsigned)ix >= (unsigned)g.nx) { ++ncx; ix = wrapi(ix, g.nx); }
                    if ((unsigned)iy >= (unsigned)g.ny) { ++ncy; iy = wrapi(iy, g.ny); }
                    if ((unsigned)iz >= (unsigned)g.nz) { ++ncz; iz = wrapi(iz, g.nz); }
                    cur.ox = nxo; cur.oy = nyo; cur.oz = nzo;
                    cur.cell = pack_cell(ix, iy, iz);
                    if (a.with_energy) {
                        ke = fmaf(cur.vx, cur.vx, fmaf(cur.vy, cur.vy, fmaf(cur.vz, cur.vz, ke)));
                        px += cur.vx; py += cur.vy; pz += cur.vz;
                    }
                }
            }
            if (ok && kDeposit) {
                fixed_weights(a.weights, cur.ox, cur.oy, cur.oz, w);
                dkey = box.key(ix, iy, iz);
                if (dkey < 0) {
                    deposit_global_fixed(g, a.wsum + (int64_t)sp * g.ncell, ix, iy, iz, w);
                    if (!kGather) ++nout;
                }
            }
            if (kMove && ok) {
                p.cell[i] = cur.cell;
                p.ox[i] = cur.ox; p.oy[i] = cur.oy; p.oz[i] = cur.oz;
                p.vx[i] = cur.vx; p.vy[i] = cur.vy; p.vz[i] = cur.vz;
            }
        }
        if (kDeposit) warp_run_deposit<DEP>(dkey, w, slo, shi, box.sx, box.sxy);
        i = inext;
        valid = vnext;
        cur = nxt;
    }
    if (kDeposit && box.on) {
        __syncthreads();
        flush_f32(a, it, slo, shi);
    }
    if (kMove || kGather) flush_diag<float>(a, sp, ncx, ncy, ncz, nout, ke, px, py, pz);
}

}  // namespace

template <typename P>
static void launch_k(ohpic_ctx *c, void (*kernel)(TileArgs, P, const CUtensorMap), const TileArgs &a,
                     int64_t blocks, size_t smem, const P &parts)
{
    if (blocks <= 0) return;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kernel<<<(unsigned)blocks, 256, smem, c->stream>>>(a, parts, c->emap);
    ++c->launches;
}

void launch_tiled_f32(ohpic_ctx *c, const TileArgs &a, int mode, int64_t blocks, size_t smem)
{
    const PartF32 &pp = c->p32[c->cur];
    switch (mode) {
    case MODE_PUSH:
        if (a.deposit == OHPIC_DEPOSIT_MATCH)
            launch_k(c, tiled_f32<MODE_PUSH, OHPIC_DEPOSIT_MATCH>, a, blocks, smem, pp);
        else if (a.deposit == OHPIC_DEPOSIT_UNIFORM)
            launch_k(c, tiled_f32<MODE_PUSH, OHPIC_DEPOSIT_UNIFORM>, a, blocks, smem, pp);
        else launch_k(c, tiled_f32<MODE_PUSH, OHPIC_DEPOSIT_RUNS>, a, blocks, smem, pp);
        break;
    case MODE_DEPOSIT:
        if (a.deposit == OHPIC_DEPOSIT_MATCH)
            launch_k(c, tiled_f32<MODE_DEPOSIT, OHPIC_DEPOSIT_MATCH>, a, blocks, smem, pp);
        else if (a.deposit == OHPIC_DEPOSIT_UNIFORM)
            launch_k(c, tiled_f32<MODE_DEPOSIT, OHPIC_DEPOSIT_UNIFORM>, a, blocks, smem, pp);
        else launch_k(c, tiled_f32<MODE_DEPOSIT, OHPIC_DEPOSIT_RUNS>, a, blocks, smem, pp);
        break;
    case MODE_MOVE: launch_k(c, tiled_f32<MODE_MOVE, OHPIC_DEPOSIT_RUNS>, a, blocks, smem, pp); break;
    case MODE_INTERP: launch_k(c, tiled_f32<MODE_INTERP, OHPIC_DEPOSIT_RUNS>, a, blocks, smem, pp); break;
    }
}

}  // namespace ohpic
