// particles.cu -- tiled particle kernels: fused gather + Boris + periodic wrap +
// CIC deposit, and the gather-only / deposit-only / move-only variants.
//
// Reference path (per particle, src/ohhelppic3d.f90:311-358):
//   scatter   src/scatter/linear_scatter.f90:32-53
//   interp    src/interpolator/linear_interpolator.f90:33-67
//   move      src/particle_mover/particle_mover_boris.f90:37-62
//   boundary  src/particle_boundary/periodic_particle_boundary.f90:42-53 (twice)
//
// Work decomposition.  Particles of each species are kept sorted by tile-major
// cell index (sort.cu), so the particles of one tile are one contiguous range.
// One CTA takes (species, tile, part): it stages the tile's node E field plus a
// halo of `halo` cells into shared memory, zeroes a shared rho tile of the same
// extent, streams its particles with 16-byte vector loads and stores (2 FP64
// or 4 FP32 particles per thread per iteration), and flushes the rho tile to
// global memory once.  Particles that drifted outside the staged box since the
// last sort gather from / deposit to global memory instead.  Deposits into the
// shared tile are first summed in registers over a thread's particles when they
// share a cell, then across the lanes of a warp that share a cell
// (__match_any_sync + a log-step tree), so one lane issues the 8 shared atomics
// of each distinct cell.
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

constexpr unsigned kFull = 0xffffffffu;

template <typename T> struct V4;
template <> struct V4<float> { using type = float4; };
template <> struct V4<double> { using type = dnode; };

// Read-only global loads of one E node.
__device__ __forceinline__ float4 ldg_node(const float4 *p) { return __ldg(p); }
__device__ __forceinline__ dnode ldg_node(const dnode *p)
{
    const double2 a = __ldg((const double2 *)p), b = __ldg((const double2 *)p + 1);
    dnode r;
    r.x = a.x; r.y = a.y; r.z = b.x; r.w = b.y;
    return r;
}

__device__ __forceinline__ void flag_error(DevDiag *d, int code, int info)
{
    if (atomicCAS(&d->err_code, 0, code) == 0) d->err_info = info;
}

// CIC weights of node floor(x) (w0) and floor(x)+1 (w1); see the header for D1.
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

// Periodic tile-relative cell offset; true when cells d and d+1 lie in the staged box.
__device__ __forceinline__ int rel_cell(int i, int o, int n, int t, int h)
{
    int d = i - o;
    if (d >= t + h) d -= n;
    else if (d < -h) d += n;
    return d;
}

__device__ __forceinline__ int wrapi(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

// Sum w[0..7] over the lanes that hold the same key; the lowest such lane ends
// with the group total (the tree of "Voting and shuffling to optimize atomic
// operations", NVIDIA developer blog, 2015).  All 32 lanes must call this.
template <typename T>
__device__ __forceinline__ bool reduce_peers(int key, T w[8])
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned peers = __match_any_sync(kFull, key);
    unsigned rel = __popc(peers & ((1u << lane) - 1u));
    const bool leader = rel == 0;
    unsigned higher = peers & ~((2u << lane) - 1u);
    while (__any_sync(kFull, higher != 0)) {
        const int next = __ffs(higher);
        const int src = next ? next - 1 : (int)lane;
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            T t = __shfl_sync(kFull, w[v], src);
            if (next) w[v] += t;
        }
        higher &= ~__ballot_sync(kFull, rel & 1u);
        rel >>= 1;
    }
    return leader;
}

__device__ __forceinline__ void atomic_add_t(float *p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_t(double *p, double v) { atomicAdd(p, v); }

// Deposits the contribution (key = staged node-box index of the cell's low
// corner, or <0 for none) of every lane after warp aggregation.
template <typename T>
__device__ __forceinline__ void deposit_shared(int key, T w[8], T *srho, int sx, int sxy)
{
    const int k = key >= 0 ? key : -1 - (int)(threadIdx.x & 31u);
    const bool leader = reduce_peers(k, w);
    if (leader && key >= 0) {
        T *b = srho + key;
        atomic_add_t(b, w[0]);
        atomic_add_t(b + 1, w[1]);
        atomic_add_t(b + sx, w[2]);
        atomic_add_t(b + sx + 1, w[3]);
        atomic_add_t(b + sxy, w[4]);
        atomic_add_t(b + sxy + 1, w[5]);
        atomic_add_t(b + sxy + sx, w[6]);
        atomic_add_t(b + sxy + sx + 1, w[7]);
    }
}

template <typename T>
__device__ __forceinline__ void deposit_global(const Geom &g, T *rho, int ix, int iy, int iz,
                                               const T w[8])
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

template <int PPT>
__device__ __forceinline__ bool get_item(const TileArgs &a, Item &it)
{
    const int64_t b = blockIdx.x;
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

// ---------------------------------------------------------------------------
// Shared-memory staging.
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void stage_tile(const TileArgs &a, const Item &it, typename V4<T>::type *sE,
                                           T *srho, bool need_e, bool need_rho)
{
    using Vec = typename V4<T>::type;
    const Geom &g = a.g;
    const int s3 = g.sx * g.sy * g.sz;
    const Vec *E = (const Vec *)a.epad;
    for (int i = threadIdx.x; i < s3; i += blockDim.x) {
        if (need_e) {
            const int ax = i % g.sx, by = (i / g.sx) % g.sy, cz = i / (g.sx * g.sy);
            sE[i] = E[((int64_t)(it.z0 + cz) * g.gy + (it.y0 + by)) * g.gx + (it.x0 + ax)];
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

// Gathers E at a cell from the staged box (d* = tile-relative cell) or from global memory.
template <typename T>
__device__ __forceinline__ void load_nodes(const TileArgs &a, bool inside, int dx, int dy, int dz, int ix,
                                           int iy, int iz, const typename V4<T>::type *sE,
                                           typename V4<T>::type nd[8])
{
    using Vec = typename V4<T>::type;
    const Geom &g = a.g;
    if (inside) {
        const int sxy = g.sx * g.sy;
        const Vec *b = sE + (dx + g.halo) + g.sx * (dy + g.halo) + sxy * (dz + g.halo);
        nd[0] = b[0];
        nd[1] = b[1];
        nd[2] = b[g.sx];
        nd[3] = b[g.sx + 1];
        nd[4] = b[sxy];
        nd[5] = b[sxy + 1];
        nd[6] = b[sxy + g.sx];
        nd[7] = b[sxy + g.sx + 1];
    } else {
        const Vec *E = (const Vec *)a.epad;
        const int64_t gxy = (int64_t)g.gx * g.gy;
        const Vec *b = E + (ix + g.halo) + (int64_t)g.gx * (iy + g.halo) + gxy * (iz + g.halo);
        nd[0] = ldg_node(b);
        nd[1] = ldg_node(b + 1);
        nd[2] = ldg_node(b + g.gx);
        nd[3] = ldg_node(b + g.gx + 1);
        nd[4] = ldg_node(b + gxy);
        nd[5] = ldg_node(b + gxy + 1);
        nd[6] = ldg_node(b + gxy + g.gx);
        nd[7] = ldg_node(b + gxy + g.gx + 1);
    }
}

// Block-wide reduction of the per-thread diagnostics into DevDiag.
template <typename T>
__device__ void flush_diag(const TileArgs &a, int sp, unsigned cx, unsigned cy, unsigned cz, unsigned outside,
                           T ke, T px, T py, T pz)
{
    __shared__ double red[8][32];
    double v[8] = {(double)cx, (double)cy, (double)cz, (double)outside, (double)ke, (double)px, (double)py,
                   (double)pz};
#pragma unroll
    for (int k = 0; k < 8; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(kFull, v[k], o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < 8; ++k) red[k][warp] = v[k];
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        for (int k = 0; k < 8; ++k) {
            double s = lane < nw ? red[k][lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
            v[k] = s;
        }
        if (lane == 0) {
            DevDiag *d = a.diag;
            if (v[0] != 0.0) atomicAdd(&d->crossings[0], (unsigned long long)v[0]);
            if (v[1] != 0.0) atomicAdd(&d->crossings[1], (unsigned long long)v[1]);
            if (v[2] != 0.0) atomicAdd(&d->crossings[2], (unsigned long long)v[2]);
            if (v[3] != 0.0) atomicAdd(&d->outside, (unsigned long long)v[3]);
            if (a.with_energy) {
                atomicAdd(&d->kin[sp][0], v[4]);
                atomicAdd(&d->kin[sp][1], v[5]);
                atomicAdd(&d->kin[sp][2], v[6]);
                atomicAdd(&d->kin[sp][3], v[7]);
            }
        }
    }
}

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

// ===========================================================================
// FP64 form: 2 particles per thread (double2 loads/stores).
// ===========================================================================
template <int MODE, bool STRICT>
__global__ void __launch_bounds__(256) tiled_f64(TileArgs a, PartF64 p)
{
    constexpr int PPT = 2;
    using Ops = typename std::conditional<STRICT, StrictOps, FastOps>::type;
    constexpr bool kGather = MODE != MODE_DEPOSIT;
    constexpr bool kMove = MODE == MODE_PUSH || MODE == MODE_MOVE;
    constexpr bool kDeposit = MODE == MODE_PUSH || MODE == MODE_DEPOSIT;

    Item it;
    if (!get_item<PPT>(a, it)) return;
    const Geom &g = a.g;
    const bool staged = it.tile >= 0;
    extern __shared__ __align__(16) unsigned char smem[];
    const int s3 = g.sx * g.sy * g.sz;
    dnode *sE = (dnode *)smem;
    double *srho = (double *)(smem + (kGather ? (size_t)s3 * sizeof(dnode) : 0));
    if (staged) {
        stage_tile<double>(a, it, sE, srho, kGather, kDeposit);
        __syncthreads();
    }

    const int sp = it.sp;
    const SpeciesConst &c = a.sc[sp];
    const int64_t end = a.seg[sp] + a.count[sp];
    const int sxy = g.sx * g.sy;
    unsigned ncx = 0, ncy = 0, ncz = 0, nout = 0;
    double ke = 0.0, px = 0.0, py = 0.0, pz = 0.0;

    for (int64_t grp = it.g0 + threadIdx.x; grp - threadIdx.x < it.g1; grp += blockDim.x) {
        const bool gvalid = grp < it.g1;
        const int64_t i0 = grp * PPT;
        double X[PPT], Y[PPT], Z[PPT], VX[PPT], VY[PPT], VZ[PPT];
        if (gvalid) {
            double2 t;
            t = *(const double2 *)(p.x + i0); X[0] = t.x; X[1] = t.y;
            t = *(const double2 *)(p.y + i0); Y[0] = t.x; Y[1] = t.y;
            t = *(const double2 *)(p.z + i0); Z[0] = t.x; Z[1] = t.y;
            if (kGather) {
                t = *(const double2 *)(p.vx + i0); VX[0] = t.x; VX[1] = t.y;
                t = *(const double2 *)(p.vy + i0); VY[0] = t.x; VY[1] = t.y;
                t = *(const double2 *)(p.vz + i0); VZ[0] = t.x; VZ[1] = t.y;
            }
        }
        int key[PPT];
        double w[PPT][8];
        int cx[PPT], cy[PPT], cz[PPT];
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            const bool valid = gvalid && (i0 + j) < end;
            key[j] = -1;
            if (!valid) continue;
            double x = X[j], y = Y[j], z = Z[j];
            if (kGather) {
                const int ix = (int)x, iy = (int)y, iz = (int)z;
                if ((unsigned)ix >= (unsigned)g.nx || (unsigned)iy >= (unsigned)g.ny ||
                    (unsigned)iz >= (unsigned)g.nz) {
                    flag_error(a.diag, OHPIC_ERR_BOUNDS, 1);
                    continue;
                }
                const int dx = rel_cell(ix, it.x0, g.nx, g.tx, g.halo);
                const int dy = rel_cell(iy, it.y0, g.ny, g.ty, g.halo);
                const int dz = rel_cell(iz, it.z0, g.nz, g.tz, g.halo);
                const bool inside = staged && (unsigned)(dx + g.halo) < (unsigned)(g.tx + 2 * g.halo) &&
                                    (unsigned)(dy + g.halo) < (unsigned)(g.ty + 2 * g.halo) &&
                                    (unsigned)(dz + g.halo) < (unsigned)(g.tz + 2 * g.halo);
                nout += !inside;
                dnode nd[8];
                load_nodes<double>(a, inside, dx, dy, dz, ix, iy, iz, sE, nd);
                double wx0, wx1, wy0, wy1, wz0, wz1;
                cic<double>(a.weights, Ops::sub(x, (double)ix), wx0, wx1);
                cic<double>(a.weights, Ops::sub(y, (double)iy), wy0, wy1);
                cic<double>(a.weights, Ops::sub(z, (double)iz), wz0, wz1);
                double ex, ey, ez;
                if (STRICT) {
                    // ret = ret + v*rx*ry*rz, i (x) outermost (linear_interpolator.f90:62-66).
                    const double wxs[2] = {wx0, wx1}, wys[2] = {wy0, wy1}, wzs[2] = {wz0, wz1};
                    ex = 0.0; ey = 0.0; ez = 0.0;
#pragma unroll
                    for (int ii = 0; ii < 2; ++ii)
#pragma unroll
                        for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                            for (int kk = 0; kk < 2; ++kk) {
                                const dnode v = nd[ii + 2 * jj + 4 * kk];
                                ex = Ops::add(ex, Ops::mul(Ops::mul(Ops::mul(v.x, wxs[ii]), wys[jj]), wzs[kk]));
                                ey = Ops::add(ey, Ops::mul(Ops::mul(Ops::mul(v.y, wxs[ii]), wys[jj]), wzs[kk]));
                                ez = Ops::add(ez, Ops::mul(Ops::mul(Ops::mul(v.z, wxs[ii]), wys[jj]), wzs[kk]));
                            }
                } else {
                    const double a00 = wx0 * wy0, a10 = wx1 * wy0, a01 = wx0 * wy1, a11 = wx1 * wy1;
                    const double ww[8] = {a00 * wz0, a10 * wz0, a01 * wz0, a11 * wz0,
                                          a00 * wz1, a10 * wz1, a01 * wz1, a11 * wz1};
                    ex = 0.0; ey = 0.0; ez = 0.0;
#pragma unroll
                    for (int n = 0; n < 8; ++n) {
                        ex = fma(nd[n].x, ww[n], ex);
                        ey = fma(nd[n].y, ww[n], ey);
                        ez = fma(nd[n].z, ww[n], ez);
                    }
                }
                if (MODE == MODE_INTERP) {
                    double *o = a.interp_out + 3 * (i0 + j);
                    o[0] = ex;
                    o[1] = ey;
                    o[2] = ez;
                }
                if (kMove) {
                    // Boris (particle_mover_boris.f90:42-56); t and s are per-species constants.
                    const double qm = c.qm, dt2 = c.dt2;
                    const double upm0 = Ops::add(VX[j], Ops::mul(Ops::mul(qm, ex), dt2));
                    const double upm1 = Ops::add(VY[j], Ops::mul(Ops::mul(qm, ey), dt2));
                    const double upm2 = Ops::add(VZ[j], Ops::mul(Ops::mul(qm, ez), dt2));
                    const double upa0 = Ops::add(upm0, Ops::sub(Ops::mul(upm1, c.t[2]), Ops::mul(upm2, c.t[1])));
                    const double upa1 = Ops::add(upm1, Ops::sub(Ops::mul(upm2, c.t[0]), Ops::mul(upm0, c.t[2])));
                    const double upa2 = Ops::add(upm2, Ops::sub(Ops::mul(upm0, c.t[1]), Ops::mul(upm1, c.t[0])));
                    const double upp0 = Ops::add(upm0, Ops::sub(Ops::mul(upa1, c.s[2]), Ops::mul(upa2, c.s[1])));
                    const double upp1 = Ops::add(upm1, Ops::sub(Ops::mul(upa2, c.s[0]), Ops::mul(upa0, c.s[2])));
                    const double upp2 = Ops::add(upm2, Ops::sub(Ops::mul(upa0, c.s[1]), Ops::mul(upa1, c.s[0])));
                    VX[j] = Ops::add(upp0, Ops::mul(Ops::mul(qm, ex), dt2));
                    VY[j] = Ops::add(upp1, Ops::mul(Ops::mul(qm, ey), dt2));
                    VZ[j] = Ops::add(upp2, Ops::mul(Ops::mul(qm, ez), dt2));
                    // Position (:60-62) and the periodic boundary applied twice.
                    x = Ops::add(x, Ops::mul(VX[j], c.dt));
                    y = Ops::add(y, Ops::mul(VY[j], c.dt));
                    z = Ops::add(z, Ops::mul(VZ[j], c.dt));
                    const double fnx = (double)g.nx, fny = (double)g.ny, fnz = (double)g.nz;
                    ncx += (x < 0.0 || x >= fnx);
                    ncy += (y < 0.0 || y >= fny);
                    ncz += (z < 0.0 || z >= fnz);
#pragma unroll
                    for (int rep = 0; rep < 2; ++rep) {
                        if (x < 0.0) x = Ops::add(fnx, x);
                        if (x >= fnx) x = Ops::sub(x, fnx);
                        if (y < 0.0) y = Ops::add(fny, y);
                        if (y >= fny) y = Ops::sub(y, fny);
                        if (z < 0.0) z = Ops::add(fnz, z);
                        if (z >= fnz) z = Ops::sub(z, fnz);
                    }
                    X[j] = x; Y[j] = y; Z[j] = z;
                    if (a.with_energy) {
                        ke = fma(VX[j], VX[j], fma(VY[j], VY[j], fma(VZ[j], VZ[j], ke)));
                        px += VX[j]; py += VY[j]; pz += VZ[j];
                    }
                }
            }
            if (kDeposit) {
                const int jx = (int)x, jy = (int)y, jz = (int)z;
                if ((unsigned)jx >= (unsigned)g.nx || (unsigned)jy >= (unsigned)g.ny ||
                    (unsigned)jz >= (unsigned)g.nz) {
                    flag_error(a.diag, OHPIC_ERR_BOUNDS, 2);
                    continue;
                }
                double wx0, wx1, wy0, wy1, wz0, wz1;
                cic<double>(a.weights, x - (double)jx, wx0, wx1);
                cic<double>(a.weights, y - (double)jy, wy0, wy1);
                cic<double>(a.weights, z - (double)jz, wz0, wz1);
                // amount*rx*ry*rz (linear_scatter.f90:47-49), factored without changing rounding.
                const double q0 = c.q * wx0, q1 = c.q * wx1;
                const double b00 = q0 * wy0, b10 = q1 * wy0, b01 = q0 * wy1, b11 = q1 * wy1;
                w[j][0] = b00 * wz0; w[j][1] = b10 * wz0; w[j][2] = b01 * wz0; w[j][3] = b11 * wz0;
                w[j][4] = b00 * wz1; w[j][5] = b10 * wz1; w[j][6] = b01 * wz1; w[j][7] = b11 * wz1;
                const int dx = rel_cell(jx, it.x0, g.nx, g.tx, g.halo);
                const int dy = rel_cell(jy, it.y0, g.ny, g.ty, g.halo);
                const int dz = rel_cell(jz, it.z0, g.nz, g.tz, g.halo);
                const bool inside = staged && (unsigned)(dx + g.halo) < (unsigned)(g.tx + 2 * g.halo) &&
                                    (unsigned)(dy + g.halo) < (unsigned)(g.ty + 2 * g.halo) &&
                                    (unsigned)(dz + g.halo) < (unsigned)(g.tz + 2 * g.halo);
                if (inside) {
                    key[j] = (dx + g.halo) + g.sx * (dy + g.halo) + sxy * (dz + g.halo);
                } else {
                    deposit_global<double>(g, (double *)a.rho, jx, jy, jz, w[j]);
                    if (!kGather) ++nout;
                }
                cx[j] = jx; cy[j] = jy; cz[j] = jz;
            }
            X[j] = x; Y[j] = y; Z[j] = z;
        }
        if (kDeposit) {
            // Register pre-sum when both particles of the thread share a cell.
            if (key[0] >= 0 && key[0] == key[1]) {
#pragma unroll
                for (int v = 0; v < 8; ++v) w[0][v] += w[1][v];
                key[1] = -1;
            }
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                if (!__any_sync(kFull, key[j] >= 0)) continue;
                deposit_shared<double>(key[j], w[j], srho, g.sx, sxy);
            }
        }
        if (kMove && gvalid) {
            *(double2 *)(p.x + i0) = make_double2(X[0], X[1]);
            *(double2 *)(p.y + i0) = make_double2(Y[0], Y[1]);
            *(double2 *)(p.z + i0) = make_double2(Z[0], Z[1]);
            *(double2 *)(p.vx + i0) = make_double2(VX[0], VX[1]);
            *(double2 *)(p.vy + i0) = make_double2(VY[0], VY[1]);
            *(double2 *)(p.vz + i0) = make_double2(VZ[0], VZ[1]);
        }
        (void)cx; (void)cy; (void)cz;
    }
    if (kDeposit && staged) {
        __syncthreads();
        flush_tile<double>(a, it, srho);
    }
    if (kMove || kGather) flush_diag<double>(a, sp, ncx, ncy, ncz, nout, ke, px, py, pz);
}

// ===========================================================================
// FP32 form: 4 particles per thread (int4/float4 loads/stores).
// ===========================================================================
template <int MODE>
__global__ void __launch_bounds__(256) tiled_f32(TileArgs a, PartF32 p)
{
    constexpr int PPT = 4;
    constexpr bool kGather = MODE != MODE_DEPOSIT;
    constexpr bool kMove = MODE == MODE_PUSH || MODE == MODE_MOVE;
    constexpr bool kDeposit = MODE == MODE_PUSH || MODE == MODE_DEPOSIT;

    Item it;
    if (!get_item<PPT>(a, it)) return;
    const Geom &g = a.g;
    const bool staged = it.tile >= 0;
    extern __shared__ __align__(16) unsigned char smem[];
    const int s3 = g.sx * g.sy * g.sz;
    float4 *sE = (float4 *)smem;
    float *srho = (float *)(smem + (kGather ? (size_t)s3 * sizeof(float4) : 0));
    if (staged) {
        stage_tile<float>(a, it, sE, srho, kGather, kDeposit);
        __syncthreads();
    }

    const int sp = it.sp;
    const SpeciesConst &c = a.sc[sp];
    const float qm = (float)c.qm, dt2 = (float)c.dt2, dtf = (float)c.dt, qf = (float)c.q;
    const float t0 = (float)c.t[0], t1 = (float)c.t[1], t2 = (float)c.t[2];
    const float s0 = (float)c.s[0], s1 = (float)c.s[1], s2 = (float)c.s[2];
    const int64_t end = a.seg[sp] + a.count[sp];
    const int sxy = g.sx * g.sy;
    unsigned ncx = 0, ncy = 0, ncz = 0, nout = 0;
    float ke = 0.f, px = 0.f, py = 0.f, pz = 0.f;

    for (int64_t grp = it.g0 + threadIdx.x; grp - threadIdx.x < it.g1; grp += blockDim.x) {
        const bool gvalid = grp < it.g1;
        const int64_t i0 = grp * PPT;
        int4 C4 = make_int4(0, 0, 0, 0);
        float4 OX = make_float4(0, 0, 0, 0), OY = OX, OZ = OX, VX = OX, VY = OX, VZ = OX;
        if (gvalid) {
            C4 = *(const int4 *)(p.cell + i0);
            OX = *(const float4 *)(p.ox + i0);
            OY = *(const float4 *)(p.oy + i0);
            OZ = *(const float4 *)(p.oz + i0);
            if (kGather) {
                VX = *(const float4 *)(p.vx + i0);
                VY = *(const float4 *)(p.vy + i0);
                VZ = *(const float4 *)(p.vz + i0);
            }
        }
        int *Cc = (int *)&C4;
        float *ox = (float *)&OX, *oy = (float *)&OY, *oz = (float *)&OZ;
        float *vx = (float *)&VX, *vy = (float *)&VY, *vz = (float *)&VZ;
        int key[PPT];
        float w[PPT][8];
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            const bool valid = gvalid && (i0 + j) < end;
            key[j] = -1;
            if (!valid) continue;
            int ix = cell_x(Cc[j]), iy = cell_y(Cc[j]), iz = cell_z(Cc[j]);
            if (ix >= g.nx || iy >= g.ny || iz >= g.nz) {
                flag_error(a.diag, OHPIC_ERR_BOUNDS, 3);
                continue;
            }
            if (kGather) {
                const int dx = rel_cell(ix, it.x0, g.nx, g.tx, g.halo);
                const int dy = rel_cell(iy, it.y0, g.ny, g.ty, g.halo);
                const int dz = rel_cell(iz, it.z0, g.nz, g.tz, g.halo);
                const bool inside = staged && (unsigned)(dx + g.halo) < (unsigned)(g.tx + 2 * g.halo) &&
                                    (unsigned)(dy + g.halo) < (unsigned)(g.ty + 2 * g.halo) &&
                                    (unsigned)(dz + g.halo) < (unsigned)(g.tz + 2 * g.halo);
                nout += !inside;
                float4 nd[8];
                load_nodes<float>(a, inside, dx, dy, dz, ix, iy, iz, sE, nd);
                float wx0, wx1, wy0, wy1, wz0, wz1;
                cic<float>(a.weights, ox[j], wx0, wx1);
                cic<float>(a.weights, oy[j], wy0, wy1);
                cic<float>(a.weights, oz[j], wz0, wz1);
                const float a00 = wx0 * wy0, a10 = wx1 * wy0, a01 = wx0 * wy1, a11 = wx1 * wy1;
                const float ww[8] = {a00 * wz0, a10 * wz0, a01 * wz0, a11 * wz0,
                                     a00 * wz1, a10 * wz1, a01 * wz1, a11 * wz1};
                float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll
                for (int n = 0; n < 8; ++n) {
                    ex = fmaf(nd[n].x, ww[n], ex);
                    ey = fmaf(nd[n].y, ww[n], ey);
                    ez = fmaf(nd[n].z, ww[n], ez);
                }
                if (MODE == MODE_INTERP) {
                    double *o = a.interp_out + 3 * (i0 + j);
                    o[0] = ex;
                    o[1] = ey;
                    o[2] = ez;
                }
                if (kMove) {
                    const float hx = qm * ex * dt2, hy = qm * ey * dt2, hz = qm * ez * dt2;
                    const float um0 = vx[j] + hx, um1 = vy[j] + hy, um2 = vz[j] + hz;
                    const float ua0 = um0 + (um1 * t2 - um2 * t1);
                    const float ua1 = um1 + (um2 * t0 - um0 * t2);
                    const float ua2 = um2 + (um0 * t1 - um1 * t0);
                    const float up0 = um0 + (ua1 * s2 - ua2 * s1);
                    const float up1 = um1 + (ua2 * s0 - ua0 * s2);
                    const float up2 = um2 + (ua0 * s1 - ua1 * s0);
                    vx[j] = up0 + hx;
                    vy[j] = up1 + hy;
                    vz[j] = up2 + hz;
                    // Offset update in cell units; crossings move the integer cell and wrap it.
                    float nxo = fmaf(vx[j], dtf, ox[j]);
                    float nyo = fmaf(vy[j], dtf, oy[j]);
                    float nzo = fmaf(vz[j], dtf, oz[j]);
                    float fx = floorf(nxo), fy = floorf(nyo), fz = floorf(nzo);
                    nxo -= fx; nyo -= fy; nzo -= fz;
                    if (nxo >= 1.f) { nxo = 0.f; fx += 1.f; }
                    if (nyo >= 1.f) { nyo = 0.f; fy += 1.f; }
                    if (nzo >= 1.f) { nzo = 0.f; fz += 1.f; }
                    ix += (int)fx; iy += (int)fy; iz += (int)fz;
                    if ((unsigned)ix >= (unsigned)g.nx) { ++ncx; ix = wrapi(ix, g.nx); }
                    if ((unsigned)iy >= (unsigned)g.ny) { ++ncy; iy = wrapi(iy, g.ny); }
                    if ((unsigned)iz >= (unsigned)g.nz) { ++ncz; iz = wrapi(iz, g.nz); }
                    ox[j] = nxo; oy[j] = nyo; oz[j] = nzo;
                    Cc[j] = pack_cell(ix, iy, iz);
                    if (a.with_energy) {
                        ke = fmaf(vx[j], vx[j], fmaf(vy[j], vy[j], fmaf(vz[j], vz[j], ke)));
                        px += vx[j]; py += vy[j]; pz += vz[j];
                    }
                }
            }
            if (kDeposit) {
                float wx0, wx1, wy0, wy1, wz0, wz1;
                cic<float>(a.weights, ox[j], wx0, wx1);
                cic<float>(a.weights, oy[j], wy0, wy1);
                cic<float>(a.weights, oz[j], wz0, wz1);
                const float q0 = qf * wx0, q1 = qf * wx1;
                const float b00 = q0 * wy0, b10 = q1 * wy0, b01 = q0 * wy1, b11 = q1 * wy1;
                w[j][0] = b00 * wz0; w[j][1] = b10 * wz0; w[j][2] = b01 * wz0; w[j][3] = b11 * wz0;
                w[j][4] = b00 * wz1; w[j][5] = b10 * wz1; w[j][6] = b01 * wz1; w[j][7] = b11 * wz1;
                const int dx = rel_cell(ix, it.x0, g.nx, g.tx, g.halo);
                const int dy = rel_cell(iy, it.y0, g.ny, g.ty, g.halo);
                const int dz = rel_cell(iz, it.z0, g.nz, g.tz, g.halo);
                const bool inside = staged && (unsigned)(dx + g.halo) < (unsigned)(g.tx + 2 * g.halo) &&
                                    (unsigned)(dy + g.halo) < (unsigned)(g.ty + 2 * g.halo) &&
                                    (unsigned)(dz + g.halo) < (unsigned)(g.tz + 2 * g.halo);
                if (inside) {
                    key[j] = (dx + g.halo) + g.sx * (dy + g.halo) + sxy * (dz + g.halo);
                } else {
                    deposit_global<float>(g, (float *)a.rho, ix, iy, iz, w[j]);
                    if (!kGather) ++nout;
                }
            }
        }
        if (kDeposit) {
            // Register pre-sum over the thread's particles that share the first cell.
            bool uniform = key[0] >= 0;
#pragma unroll
            for (int j = 1; j < PPT; ++j) uniform = uniform && key[j] == key[0];
            if (uniform) {
#pragma unroll
                for (int j = 1; j < PPT; ++j) {
#pragma unroll
                    for (int v = 0; v < 8; ++v) w[0][v] += w[j][v];
                    key[j] = -1;
                }
            }
#pragma unroll
            for (int j = 0; j < PPT; ++j) {
                if (!__any_sync(kFull, key[j] >= 0)) continue;
                deposit_shared<float>(key[j], w[j], srho, g.sx, sxy);
            }
        }
        if (kMove && gvalid) {
            *(int4 *)(p.cell + i0) = C4;
            *(float4 *)(p.ox + i0) = OX;
            *(float4 *)(p.oy + i0) = OY;
            *(float4 *)(p.oz + i0) = OZ;
            *(float4 *)(p.vx + i0) = VX;
            *(float4 *)(p.vy + i0) = VY;
            *(float4 *)(p.vz + i0) = VZ;
        }
    }
    if (kDeposit && staged) {
        __syncthreads();
        flush_tile<float>(a, it, srho);
    }
    if (kMove || kGather) flush_diag<float>(a, sp, ncx, ncy, ncz, nout, ke, px, py, pz);
}

// ---------------------------------------------------------------------------
// Conversions between the host's FP64 records and the device forms.
// stage holds n particles either as 6 SoA arrays of n doubles (aos = 0) or as
// AoS records of stride_doubles (aos = 1, x..vz at 0..5).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void read_stage(const double *s, int64_t i, int64_t n, int aos, int64_t stride,
                                           double r[6])
{
    if (aos) {
#pragma unroll
        for (int k = 0; k < 6; ++k) r[k] = s[i * stride + k];
    } else {
#pragma unroll
        for (int k = 0; k < 6; ++k) r[k] = s[k * n + i];
    }
}

__global__ void k_stage_to_f64(const double *stage, int64_t n, int aos, int64_t stride, PartF64 p, uint32_t *ids,
                               int64_t dst, uint32_t id0)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double r[6];
        read_stage(stage, i, n, aos, stride, r);
        const int64_t o = dst + i;
        p.x[o] = r[0]; p.y[o] = r[1]; p.z[o] = r[2];
        p.vx[o] = r[3]; p.vy[o] = r[4]; p.vz[o] = r[5];
        if (ids) ids[o] = id0 + (uint32_t)i;
    }
}

// Absolute FP64 position -> (cell, FP32 offset).  The offset is rounded to
// FP32; a value that rounds up to 1 moves to offset 0 of the next cell.
__device__ __forceinline__ void split_pos(double x, int n, int &i, float &o, DevDiag *d)
{
    int c = (int)floor(x);
    float f = (float)(x - (double)c);
    if (f >= 1.f) { f = 0.f; ++c; }
    if (c >= n) c -= n;
    if (c < 0) c += n;
    if ((unsigned)c >= (unsigned)n) {
        flag_error(d, OHPIC_ERR_BOUNDS, 4);
        c = 0;
    }
    i = c;
    o = f;
}

__global__ void k_stage_to_f32(const double *stage, int64_t n, int aos, int64_t stride, PartF32 p, uint32_t *ids,
                               int64_t dst, uint32_t id0, int nx, int ny, int nz, DevDiag *d)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double r[6];
        read_stage(stage, i, n, aos, stride, r);
        int ix, iy, iz;
        float ox, oy, oz;
        split_pos(r[0], nx, ix, ox, d);
        split_pos(r[1], ny, iy, oy, d);
        split_pos(r[2], nz, iz, oz, d);
        const int64_t o = dst + i;
        p.cell[o] = pack_cell(ix, iy, iz);
        p.ox[o] = ox; p.oy[o] = oy; p.oz[o] = oz;
        p.vx[o] = (float)r[3]; p.vy[o] = (float)r[4]; p.vz[o] = (float)r[5];
        if (ids) ids[o] = id0 + (uint32_t)i;
    }
}

// Device form -> 6 SoA arrays of n doubles (+ ids as the 7th block, reinterpreted).
__global__ void k_f64_to_stage(PartF64 p, int64_t src, int64_t n, double *stage)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = src + i;
        stage[i] = p.x[o]; stage[n + i] = p.y[o]; stage[2 * n + i] = p.z[o];
        stage[3 * n + i] = p.vx[o]; stage[4 * n + i] = p.vy[o]; stage[5 * n + i] = p.vz[o];
    }
}

__global__ void k_f32_to_stage(PartF32 p, int64_t src, int64_t n, double *stage)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = src + i;
        const int32_t c = p.cell[o];
        stage[i] = (double)cell_x(c) + (double)p.ox[o];
        stage[n + i] = (double)cell_y(c) + (double)p.oy[o];
        stage[2 * n + i] = (double)cell_z(c) + (double)p.oz[o];
        stage[3 * n + i] = p.vx[o]; stage[4 * n + i] = p.vy[o]; stage[5 * n + i] = p.vz[o];
    }
}

// Kinetic energy and momentum of every species (FP64 accumulation).
template <bool F32>
__global__ void k_kinetic(PartF64 p64, PartF32 p32, int64_t seg, int64_t n, double *out4)
{
    double ke = 0, mx = 0, my = 0, mz = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double vx, vy, vz;
        if (F32) {
            vx = p32.vx[seg + i]; vy = p32.vy[seg + i]; vz = p32.vz[seg + i];
        } else {
            vx = p64.vx[seg + i]; vy = p64.vy[seg + i]; vz = p64.vz[seg + i];
        }
        ke += vx * vx + vy * vy + vz * vz;
        mx += vx; my += vy; mz += vz;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ke += __shfl_xor_sync(kFull, ke, o);
        mx += __shfl_xor_sync(kFull, mx, o);
        my += __shfl_xor_sync(kFull, my, o);
        mz += __shfl_xor_sync(kFull, mz, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out4 + 0, ke);
        atomicAdd(out4 + 1, mx);
        atomicAdd(out4 + 2, my);
        atomicAdd(out4 + 3, mz);
    }
}

int grid_for(int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    if (b > 152 * 32) b = 152 * 32;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template <typename P>
static void launch_k(ohpic_ctx *c, void (*kernel)(TileArgs, P), const TileArgs &a, int64_t blocks, size_t smem,
                     const P &parts)
{
    if (blocks <= 0) return;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kernel<<<(unsigned)blocks, 256, smem, c->stream>>>(a, parts);
    ++c->launches;
}

void launch_tiled(ohpic_ctx *c, int mode, int strict)
{
    TileArgs a;
    a.g = c->g;
    a.nspecies = c->cfg.nspecies;
    a.weights = c->cfg.weights;
    a.split = c->split;
    a.with_energy = c->with_energy ? 1 : 0;
    a.sorted = c->sorted ? 1 : 0;
    a.chunk = 4096;
    for (int s = 0; s < OHPIC_MAX_SPECIES; ++s) {
        a.seg[s] = c->seg[s];
        a.count[s] = c->count[s];
        a.sc[s] = c->sc[s];
    }
    a.tile_begin = c->tile_begin;
    a.epad = c->epad;
    a.rho = c->rho;
    a.interp_out = c->interp_buf;
    a.diag = c->diag;

    const bool f64 = c->cfg.precision == OHPIC_FP64;
    const int PPT = f64 ? 2 : 4;
    int64_t blocks = 0;
    if (a.sorted) {
        blocks = (int64_t)a.nspecies * c->g.ntile * a.split;
    } else {
        for (int s = 0; s < a.nspecies; ++s) {
            const int64_t groups = (c->count[s] + PPT - 1) / PPT;
            blocks += (groups * PPT + a.chunk - 1) / a.chunk;
        }
    }
    const int64_t s3 = (int64_t)c->g.sx * c->g.sy * c->g.sz;
    const size_t es = f64 ? 8 : 4;
    const bool gather = mode != MODE_DEPOSIT;
    const bool dep = mode == MODE_PUSH || mode == MODE_DEPOSIT;
    size_t smem = 0;
    if (a.sorted) smem = (gather ? s3 * 4 * es : 0) + (dep ? s3 * es : 0);

    if (f64) {
        const PartF64 &pp = c->p64[c->cur];
        switch (mode * 2 + (strict ? 1 : 0)) {
        case MODE_PUSH * 2: launch_k(c, tiled_f64<MODE_PUSH, false>, a, blocks, smem, pp); break;
        case MODE_PUSH * 2 + 1: launch_k(c, tiled_f64<MODE_PUSH, true>, a, blocks, smem, pp); break;
        case MODE_MOVE * 2: launch_k(c, tiled_f64<MODE_MOVE, false>, a, blocks, smem, pp); break;
        case MODE_MOVE * 2 + 1: launch_k(c, tiled_f64<MODE_MOVE, true>, a, blocks, smem, pp); break;
        case MODE_DEPOSIT * 2:
        case MODE_DEPOSIT * 2 + 1: launch_k(c, tiled_f64<MODE_DEPOSIT, false>, a, blocks, smem, pp); break;
        case MODE_INTERP * 2: launch_k(c, tiled_f64<MODE_INTERP, false>, a, blocks, smem, pp); break;
        case MODE_INTERP * 2 + 1: launch_k(c, tiled_f64<MODE_INTERP, true>, a, blocks, smem, pp); break;
        }
    } else {
        const PartF32 &pp = c->p32[c->cur];
        switch (mode) {
        case MODE_PUSH: launch_k(c, tiled_f32<MODE_PUSH>, a, blocks, smem, pp); break;
        case MODE_MOVE: launch_k(c, tiled_f32<MODE_MOVE>, a, blocks, smem, pp); break;
        case MODE_DEPOSIT: launch_k(c, tiled_f32<MODE_DEPOSIT>, a, blocks, smem, pp); break;
        case MODE_INTERP: launch_k(c, tiled_f32<MODE_INTERP>, a, blocks, smem, pp); break;
        }
    }
}

void launch_f64_soa_from_stage(ohpic_ctx *c, const double *stage, int64_t n, int64_t dst, uint32_t id0, int aos,
                               int64_t stride_doubles)
{
    if (n <= 0) return;
    k_stage_to_f64<<<grid_for(n, 256), 256, 0, c->stream>>>(stage, n, aos, stride_doubles, c->p64[c->cur],
                                                             c->ids[c->cur], dst, id0);
    ++c->launches;
}

void launch_f64_to_f32(ohpic_ctx *c, const double *stage, int64_t n, int64_t dst, uint32_t id0, int aos,
                       int64_t stride_doubles)
{
    if (n <= 0) return;
    k_stage_to_f32<<<grid_for(n, 256), 256, 0, c->stream>>>(stage, n, aos, stride_doubles, c->p32[c->cur],
                                                             c->ids[c->cur], dst, id0, c->g.nx, c->g.ny,
                                                             c->g.nz, c->diag);
    ++c->launches;
}

void launch_to_f64_stage(ohpic_ctx *c, double *stage, int64_t src, int64_t n)
{
    if (n <= 0) return;
    if (c->cfg.precision == OHPIC_FP64)
        k_f64_to_stage<<<grid_for(n, 256), 256, 0, c->stream>>>(c->p64[c->cur], src, n, stage);
    else
        k_f32_to_stage<<<grid_for(n, 256), 256, 0, c->stream>>>(c->p32[c->cur], src, n, stage);
    ++c->launches;
}

void launch_kinetic(ohpic_ctx *c)
{
    for (int s = 0; s < c->cfg.nspecies; ++s) {
        double *out = &c->diag->kin[s][0];
        cudaMemsetAsync(out, 0, 4 * sizeof(double), c->stream);
        if (c->count[s] == 0) continue;
        if (c->cfg.precision == OHPIC_FP64)
            k_kinetic<false><<<grid_for(c->count[s], 256), 256, 0, c->stream>>>(c->p64[c->cur], c->p32[c->cur],
                                                                                 c->seg[s], c->count[s], out);
        else
            k_kinetic<true><<<grid_for(c->count[s], 256), 256, 0, c->stream>>>(c->p64[c->cur], c->p32[c->cur],
                                                                                c->seg[s], c->count[s], out);
        ++c->launches;
    }
}

}  // namespace ohpic
