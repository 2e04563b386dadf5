// tile_common.cuh -- device helpers shared by the tiled particle kernels
// (work items, the staged E/rho box, gathers, deposits, diagnostics).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

constexpr unsigned kFull = 0xffffffffu;

// Read-only global loads of one E node.
__device__ __forceinline__ float4 ldg_node(const float4 *p) { return __ldg(p); }
__device__ __forceinline__ dnode ldg_node(const dnode *p)
{
    const double2 a = __ldg((const double2 *)p), b = __ldg((const double2 *)p + 1);
    dnode r;
    r.x = a.x; r.y = a.y; r.z = b.x; r.w = b.y;
    return r;
}
__device__ __forceinline__ dnode lds_node(const dnode *p)
{
    const double2 a = ((const double2 *)p)[0], b = ((const double2 *)p)[1];
    dnode r;
    r.x = a.x; r.y = a.y; r.z = b.x; r.w = b.y;
    return r;
}
__device__ __forceinline__ float4 lds_node(const float4 *p) { return *p; }

__device__ __forceinline__ void flag_error(DevDiag *d, int code, int info)
{
    if (atomicCAS(&d->err_code, 0, code) == 0) d->err_info = info;
}

// CIC weights of node floor(x) (w0) and floor(x)+1 (w1).  The reference
// convention (linear_scatter.f90:41-42, linear_interpolator.f90:54-57) gives
// node floor(x) the weight r = x - floor(x).
template <typename T>
__device__ __forceinline__ void cic(int conv, T r, T &w0, T &w1)
{
    if (conv == OHPIC_WEIGHTS_REFERENCE) {
        w0 = r;
        w1 = T(1) - r;
    } else {
        w0 = T(1) - r;
        w1 = r;
    }
}

// The same with the convention fixed at compile time (the FP32 kernels are
// instantiated per convention: a run-time choice cost two selects per axis).
template <int CONV, typename T>
__device__ __forceinline__ void cic_c(T r, T &w0, T &w1)
{
    if (CONV == OHPIC_WEIGHTS_REFERENCE) {
        w0 = r;
        w1 = T(1) - r;
    } else {
        w0 = T(1) - r;
        w1 = r;
    }
}

__device__ __forceinline__ int wrapi(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

__device__ __forceinline__ void atomic_add_t(float *p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_t(double *p, double v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_t(unsigned long long *p, unsigned long long v) { atomicAdd(p, v); }

// 8 corner contributions of one cell into a box with row pitch sx and plane pitch sxy.
template <typename T>
__device__ __forceinline__ void add8(T *b, int sx, int sxy, const T w[8])
{
    atomic_add_t(b, w[0]);
    atomic_add_t(b + 1, w[1]);
    atomic_add_t(b + sx, w[2]);
    atomic_add_t(b + sx + 1, w[3]);
    atomic_add_t(b + sxy, w[4]);
    atomic_add_t(b + sxy + 1, w[5]);
    atomic_add_t(b + sxy + sx, w[6]);
    atomic_add_t(b + sxy + sx + 1, w[7]);
}

template <typename T>
__device__ __forceinline__ void deposit_global(const Geom &g, T *rho, int ix, int iy, int iz, const T w[8])
{
    const int ix1 = ix + 1 == g.nx ? 0 : ix + 1;
    const int iy1 = iy + 1 == g.ny ? 0 : iy + 1;
    const int iz1 = iz + 1 == g.nz ? 0 : iz + 1;
    const int64_t y0 = (int64_t)iy * g.nx, y1 = (int64_t)iy1 * g.nx;
    const int64_t z0 = (int64_t)iz * g.nx * g.ny, z1 = (int64_t)iz1 * g.nx * g.ny;
    atomic_add_t(rho + ix + y0 + z0, w[0]);
    atomic_add_t(rho + ix1 + y0 + z0, w[1]);
    atomic_add_t(rho + ix + y1 + z0, w[2]);
    atomic_add_t(rho + ix1 + y1 + z0, w[3]);
    atomic_add_t(rho + ix + y0 + z1, w[4]);
    atomic_add_t(rho + ix1 + y0 + z1, w[5]);
    atomic_add_t(rho + ix + y1 + z1, w[6]);
    atomic_add_t(rho + ix1 + y1 + z1, w[7]);
}

// ---------------------------------------------------------------------------
// Work item of a CTA.
// ---------------------------------------------------------------------------
struct Item {
    int sp;
    int tile;           // -1 when unsorted
    int64_t g0, g1;     // vector-group range [g0, g1)
    int x0, y0, z0;     // tile origin (cells)
};

// Work item b of a launch (b = blockIdx.x for a single context; the multi-run
// kernel passes the item's index within its run).
template <int PPT>
__device__ __forceinline__ bool get_item(const TileArgs &a, int64_t b, Item &it)
{
    if (a.sorted) {
        const int64_t per_sp = a.g.ntile * a.split;
        it.sp = (int)(b / per_sp);
        const int64_t r = b % per_sp;
        it.tile = (int)(r / a.split);
        const int part = (int)(r % a.split);
        const int64_t *tb = a.tile_begin + (int64_t)it.sp * (a.g.ntile + 1);
        const int64_t lo = tb[it.tile] / PPT;
        const int64_t hi = it.tile + 1 == a.g.ntile ? (tb[a.g.ntile] + PPT - 1) / PPT : tb[it.tile + 1] / PPT;
        const int64_t n = hi - lo;
        it.g0 = lo + n * part / a.split;
        it.g1 = lo + n * (part + 1) / a.split;
        const int t = it.tile;
        const int tx = t % a.g.ntx, ty = (t / a.g.ntx) % a.g.nty, tz = t / (a.g.ntx * a.g.nty);
        it.x0 = tx * a.g.tx;
        it.y0 = ty * a.g.ty;
        it.z0 = tz * a.g.tz;
    } else {
        // Unsorted: consecutive chunks of every species, no staging.
        int sp = 0;
        int64_t first = 0;
        for (; sp < a.nspecies; ++sp) {
            const int64_t groups = (a.count[sp] + PPT - 1) / PPT;
            const int64_t blocks = (groups * PPT + a.chunk - 1) / a.chunk;
            if (b < first + blocks) break;
            first += blocks;
        }
        if (sp >= a.nspecies) return false;
        it.sp = sp;
        it.tile = -1;
        const int64_t gseg = a.seg[sp] / PPT;
        const int64_t groups = (a.count[sp] + PPT - 1) / PPT;
        const int64_t gpc = a.chunk / PPT;
        it.g0 = gseg + (b - first) * gpc;
        it.g1 = min(gseg + groups, it.g0 + gpc);
        it.x0 = it.y0 = it.z0 = 0;
    }
    return true;
}

template <int PPT>
__device__ __forceinline__ bool get_item(const TileArgs &a, Item &it)
{
    return get_item<PPT>(a, (int64_t)blockIdx.x, it);
}

// Staged box: nodes (x0-halo .. x0+tx+halo) per axis, i.e. the low corners of
// cells x0-halo .. x0+tx+halo-1 ("span" cells), so a cell with box coordinate
// l in [0, span) has both its nodes inside.
struct Box {
    int ox, oy, oz;          // box origin in cells (x0 - halo, ...)
    unsigned spx, spy, spz;  // valid low-corner span per axis
    int sx, sxy;             // node pitches
    bool on;                 // staged at all
    __device__ __forceinline__ int key(int ix, int iy, int iz) const
    {
        const int lx = ix - ox, ly = iy - oy, lz = iz - oz;
        const bool in = on && (unsigned)lx < spx && (unsigned)ly < spy && (unsigned)lz < spz;
        return in ? lx + sx * ly + sxy * lz : -1;
    }
};

__device__ __forceinline__ Box make_box(const Geom &g, const Item &it)
{
    Box b;
    b.ox = it.x0 - g.halo;
    b.oy = it.y0 - g.halo;
    b.oz = it.z0 - g.halo;
    b.spx = (unsigned)(g.tx + 2 * g.halo);
    b.spy = (unsigned)(g.ty + 2 * g.halo);
    b.spz = (unsigned)(g.tz + 2 * g.halo);
    b.sx = g.sx;
    b.sxy = g.sx * g.sy;
    b.on = it.tile >= 0;
    return b;
}

template <typename NodeT, typename T>
__device__ __forceinline__ void stage_tile(const TileArgs &a, const Item &it, NodeT *sE, T *srho, bool need_e,
                                           bool need_rho)
{
    const Geom &g = a.g;
    const int s3 = g.sx * g.sy * g.sz;
    const NodeT *E = (const NodeT *)a.epad;
    for (int i = threadIdx.x; i < s3; i += blockDim.x) {
        if (need_e) {
            const int ax = i % g.sx, by = (i / g.sx) % g.sy, cz = i / (g.sx * g.sy);
            // padded index of node (x0 - halo + ax) is x0 + ax
            sE[i] = ldg_node(E + ((int64_t)(it.z0 + cz) * g.gy + (it.y0 + by)) * g.gx + (it.x0 + ax));
        }
        if (need_rho) srho[i] = T(0);
    }
}

template <typename T>
__device__ __forceinline__ void flush_tile(const TileArgs &a, const Item &it, const T *srho)
{
    const Geom &g = a.g;
    const int s3 = g.sx * g.sy * g.sz;
    T *rho = (T *)a.rho;
    for (int i = threadIdx.x; i < s3; i += blockDim.x) {
        const T v = srho[i];
        if (v != T(0)) {
            const int ax = i % g.sx, by = (i / g.sx) % g.sy, cz = i / (g.sx * g.sy);
            const int x = wrapi(it.x0 - g.halo + ax, g.nx);
            const int y = wrapi(it.y0 - g.halo + by, g.ny);
            const int z = wrapi(it.z0 - g.halo + cz, g.nz);
            atomic_add_t(rho + x + (int64_t)g.nx * (y + (int64_t)g.ny * z), v);
        }
    }
}

// E nodes of the cell with low corner (ix, iy, iz): from the staged box when key >= 0.
template <typename NodeT>
__device__ __forceinline__ void load_nodes(const TileArgs &a, const Box &b, int key, int ix, int iy, int iz,
                                           const NodeT *sE, NodeT nd[8])
{
    if (key >= 0) {
        const NodeT *p = sE + key;
        nd[0] = lds_node(p);
        nd[1] = lds_node(p + 1);
        nd[2] = lds_node(p + b.sx);
        nd[3] = lds_node(p + b.sx + 1);
        nd[4] = lds_node(p + b.sxy);
        nd[5] = lds_node(p + b.sxy + 1);
        nd[6] = lds_node(p + b.sxy + b.sx);
        nd[7] = lds_node(p + b.sxy + b.sx + 1);
    } else {
        const Geom &g = a.g;
        const NodeT *E = (const NodeT *)a.epad;
        const int64_t gxy = (int64_t)g.gx * g.gy;
        const NodeT *p = E + (ix + g.halo) + (int64_t)g.gx * (iy + g.halo) + gxy * (iz + g.halo);
        nd[0] = ldg_node(p);
        nd[1] = ldg_node(p + 1);
        nd[2] = ldg_node(p + g.gx);
        nd[3] = ldg_node(p + g.gx + 1);
        nd[4] = ldg_node(p + gxy);
        nd[5] = ldg_node(p + gxy + 1);
        nd[6] = ldg_node(p + gxy + g.gx);
        nd[7] = ldg_node(p + gxy + g.gx + 1);
    }
}

// Block-wide reduction of the per-thread diagnostics into DevDiag.  The counts
// reduce with integer warp reductions; the kinetic sums (in FP64, converted per
// thread) only when the push tracks them.  On GB300 an FP64 add runs on the narrow
// FP64 pipe, and reducing all eight tallies in FP64 at the end of every work item
// kept that pipe 4.5% busy in the FP32 push.
template <typename T>
__device__ void flush_diag(const TileArgs &a, int sp, unsigned cx, unsigned cy, unsigned cz, unsigned outside, T ke,
                           T px, T py, T pz)
{
    // The tile kernels run 256 threads (8 warps); the scratch is sized for exactly
    // that and keeps the static shared memory of a (16,8,8) tile at halo 2 within
    // two CTAs per SM.
    __shared__ unsigned cnt[4][kTileWarps];
    __shared__ double kin[4][kTileWarps];
    const bool energy = a.with_energy != 0;
    unsigned u[4] = {cx, cy, cz, outside};
#pragma unroll
    for (int k = 0; k < 4; ++k) u[k] = __reduce_add_sync(kFull, u[k]);
    double v[4] = {(double)ke, (double)px, (double)py, (double)pz};
    if (energy) {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(kFull, v[k], o);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0 && warp < kTileWarps) {
        for (int k = 0; k < 4; ++k) {
            cnt[k][warp] = u[k];
            kin[k][warp] = v[k];
        }
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = min((int)(blockDim.x >> 5), kTileWarps);
#pragma unroll
        for (int k = 0; k < 4; ++k) u[k] = __reduce_add_sync(kFull, lane < nw ? cnt[k][lane] : 0u);
        if (energy) {
            for (int k = 0; k < 4; ++k) {
                double t = lane < nw ? kin[k][lane] : 0.0;
                for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(kFull, t, o);
                v[k] = t;
            }
        }
        if (lane == 0) {
            DevDiag *d = a.diag;
            if (u[0]) atomicAdd(&d->crossings[0], (unsigned long long)u[0]);
            if (u[1]) atomicAdd(&d->crossings[1], (unsigned long long)u[1]);
            if (u[2]) atomicAdd(&d->crossings[2], (unsigned long long)u[2]);
            if (u[3]) atomicAdd(&d->outside, (unsigned long long)u[3]);
            if (energy) {
                atomicAdd(&d->kin[sp][0], v[0]);
                atomicAdd(&d->kin[sp][1], v[1]);
                atomicAdd(&d->kin[sp][2], v[2]);
                atomicAdd(&d->kin[sp][3], v[3]);
            }
        }
    }
}

// Register run of deposits into one staged cell; flushed when the cell changes.
template <typename T>
struct Run {
    int key = -1;
    T acc[8];
    __device__ __forceinline__ void add(int k, const T w[8], T *srho, int sx, int sxy)
    {
        if (k == key) {
#pragma unroll
            for (int v = 0; v < 8; ++v) acc[v] += w[v];
        } else {
            if (key >= 0) add8(srho + key, sx, sxy, acc);
            key = k;
#pragma unroll
            for (int v = 0; v < 8; ++v) acc[v] = w[v];
        }
    }
    __device__ __forceinline__ void flush(T *srho, int sx, int sxy)
    {
        if (key >= 0) add8(srho + key, sx, sxy, acc);
        key = -1;
    }
};

// Sign and ">= n" tests of a double on its bit pattern (integer ALU, not the FP64
// pipe).  lt0 is p < 0 (false for -0.0); ge is p >= n for the bits of (double)n > 0.
__device__ __forceinline__ bool lt0(double p)
{
    const long long b = __double_as_longlong(p);
    return b < 0 && b != (long long)0x8000000000000000ULL;
}
__device__ __forceinline__ bool ge_bits(double p, long long nbits) { return __double_as_longlong(p) >= nbits; }

// Strict FP64 arithmetic: every multiply and add rounds on its own, in the
// reference's operation order (no FMA contraction).
struct StrictOps {
    static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
};
struct FastOps {
    static __device__ __forceinline__ double mul(double a, double b) { return a * b; }
    static __device__ __forceinline__ double add(double a, double b) { return a + b; }
    static __device__ __forceinline__ double sub(double a, double b) { return a - b; }
};

}  // namespace
}  // namespace ohpic
