// push_f64.cu -- the plain FP64 form of the tiled particle kernels.
//
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
// halo of `halo` cells into shared memory, zeroes a shared rho box of the same
// extent, streams its particles with 16-byte vector loads and stores (two FP64
// particles per thread per iteration) and flushes the box to global memory once.  A particle whose cell lies outside the staged box (it
// drifted since the last sort, or wrapped across the periodic edge) gathers
// from and deposits to global memory instead.
//
// Deposit in fixed point.  Each particle's 8 CIC weights are integers in units
// of 2^-48 that sum to exactly 2^48: the fractional offsets are rounded to 48
// bits, and 2^48 is split axis by axis (x, then y within each half, then z
// within each quarter), each child rounded from the product of its parent and
// the axis weight and its sibling taking the difference.  The products are
// 48 x 48 -> 96-bit integer multiplies, so the weights cost no FP64 operations
// beyond the offsets; on GB300 the FP64 pipe is the bottleneck of this form.  A
// thread's consecutive particles are consecutive in cell order, so their
// weights are summed in registers while they stay in one cell and added to a
// 64-bit shared box when the cell changes; the box is flushed into per-species
// 64-bit global sums, from which the solve forms rho = sum_s q_s W_s 2^-48 in a
// fixed species order.  Integer addition is associative, so rho does not depend
// on the order in which atomics land: the FP64 form is bit-reproducible.  A
// node's sum stays below 2^64 up to 65536 particle weights per species; a flush
// that would wrap raises OHPIC_ERR_CAPACITY.
#include "f64_fixed.cuh"
#include "tile_common.cuh"

namespace ohpic {
namespace {

constexpr int kF64PerThread = 2;

__device__ __forceinline__ void add_checked(unsigned long long *p, unsigned long long v, DevDiag *d)
{
    const unsigned long long old = atomicAdd(p, v);
    if (old + v < old) flag_error(d, OHPIC_ERR_CAPACITY, 20);
}

// The 8 weights of a particle outside the staged box, straight into the global sums.
__device__ __forceinline__ void deposit_global48(const Geom &g, unsigned long long *w, int ix, int iy, int iz,
                                                 const unsigned long long u[8], DevDiag *d)
{
    const int ix1 = ix + 1 == g.nx ? 0 : ix + 1;
    const int iy1 = iy + 1 == g.ny ? 0 : iy + 1;
    const int iz1 = iz + 1 == g.nz ? 0 : iz + 1;
    const int64_t y0 = (int64_t)iy * g.nx, y1 = (int64_t)iy1 * g.nx;
    const int64_t z0 = (int64_t)iz * g.nx * g.ny, z1 = (int64_t)iz1 * g.nx * g.ny;
    add_checked(w + ix + y0 + z0, u[0], d);
    add_checked(w + ix1 + y0 + z0, u[1], d);
    add_checked(w + ix + y1 + z0, u[2], d);
    add_checked(w + ix1 + y1 + z0, u[3], d);
    add_checked(w + ix + y0 + z1, u[4], d);
    add_checked(w + ix1 + y0 + z1, u[5], d);
    add_checked(w + ix + y1 + z1, u[6], d);
    add_checked(w + ix1 + y1 + z1, u[7], d);
}

// The shared box into the species' global sums, one atomic per non-zero node.
__device__ __forceinline__ void flush_box48(const TileArgs &a, const Item &it, const unsigned long long *box)
{
    const Geom &g = a.g;
    unsigned long long *w = a.wsum + (int64_t)it.sp * g.ncell;
    const int s3 = g.sx * g.sy * g.sz;
    for (int i = threadIdx.x; i < s3; i += blockDim.x) {
        const unsigned long long v = box[i];
        if (v) {
            const int ax = i % g.sx, by = (i / g.sx) % g.sy, cz = i / (g.sx * g.sy);
            const int x = wrapi(it.x0 - g.halo + ax, g.nx);
            const int y = wrapi(it.y0 - g.halo + by, g.ny);
            const int z = wrapi(it.z0 - g.halo + cz, g.nz);
            add_checked(w + x + (int64_t)g.nx * (y + (int64_t)g.ny * z), v, a.diag);
        }
    }
}

// ===========================================================================
// FP64 form: kF64PerThread consecutive particles per thread per iteration.  Two
// (double2 vectors) spill 124 bytes per thread at two CTAs per SM; one (scalar
// loads) spills nothing but issues 38% more instructions and measured slower
// (220 against 211 ms per step at 256^3).
// ===========================================================================
// The three E components of a node (the padded node's fourth is never read).
struct d3 {
    double x, y, z;
};

__device__ __forceinline__ d3 node3(const dnode *p, bool shared)
{
    d3 r;
    if (shared) {
        const double2 a = *(const double2 *)p;
        r.x = a.x;
        r.y = a.y;
        r.z = p->z;
    } else {
        const double2 a = __ldg((const double2 *)p);
        r.x = a.x;
        r.y = a.y;
        r.z = __ldg(&p->z);
    }
    return r;
}

// E nodes of the cell with low corner (ix, iy, iz): from the staged box when key >= 0.
__device__ __forceinline__ void load_nodes3(const TileArgs &a, const Box &b, int key, int ix, int iy, int iz,
                                            const dnode *sE, d3 nd[8])
{
    const dnode *q;
    int64_t sx, sxy;
    const bool in = key >= 0;
    if (in) {
        q = sE + key;
        sx = b.sx;
        sxy = b.sxy;
    } else {
        const Geom &g = a.g;
        sx = g.gx;
        sxy = (int64_t)g.gx * g.gy;
        q = (const dnode *)a.epad + (ix + g.halo) + sx * (iy + g.halo) + sxy * (iz + g.halo);
    }
    nd[0] = node3(q, in);
    nd[1] = node3(q + 1, in);
    nd[2] = node3(q + sx, in);
    nd[3] = node3(q + sx + 1, in);
    nd[4] = node3(q + sxy, in);
    nd[5] = node3(q + sxy + 1, in);
    nd[6] = node3(q + sxy + sx, in);
    nd[7] = node3(q + sxy + sx + 1, in);
}

template <int PPT>
__device__ __forceinline__ void load_f64(const double *a, int64_t i0, double v[PPT])
{
    if constexpr (PPT == 2) {
        const double2 t = *(const double2 *)(a + i0);
        v[0] = t.x;
        v[1] = t.y;
    } else {
        v[0] = a[i0];
    }
}

template <int PPT>
__device__ __forceinline__ void store_f64(double *a, int64_t i0, const double v[PPT])
{
    if constexpr (PPT == 2) *(double2 *)(a + i0) = make_double2(v[0], v[1]);
    else a[i0] = v[0];
}

template <int MODE, bool STRICT>
__global__ void __launch_bounds__(256, 2) tiled_f64(TileArgs a, PartF64 p)
{
    constexpr int PPT = kF64PerThread;
    using Ops = typename std::conditional<STRICT, StrictOps, FastOps>::type;
    constexpr bool kGather = MODE != MODE_DEPOSIT;
    constexpr bool kMove = MODE == MODE_PUSH || MODE == MODE_MOVE;
    constexpr bool kDeposit = MODE == MODE_PUSH || MODE == MODE_DEPOSIT;

    Item it;
    if (!get_item<PPT>(a, it)) return;
    const Geom &g = a.g;
    const Box box = make_box(g, it);
    extern __shared__ __align__(32) unsigned char smem[];
    const int s3 = g.sx * g.sy * g.sz;
    dnode *sE = (dnode *)smem;
    unsigned long long *sbox = (unsigned long long *)(smem + (kGather ? (size_t)s3 * sizeof(dnode) : 0));
    if (box.on) {
        stage_tile<dnode, unsigned long long>(a, it, sE, sbox, kGather, kDeposit);
        __syncthreads();
    }

    const int sp = it.sp;
    const SpeciesConst &c = a.sc[sp];
    const int64_t end = a.seg[sp] + a.count[sp];
    const double fnx = (double)g.nx, fny = (double)g.ny, fnz = (double)g.nz;
    const long long bnx = __double_as_longlong(fnx), bny = __double_as_longlong(fny), bnz = __double_as_longlong(fnz);
    unsigned ncx = 0, ncy = 0, ncz = 0, nout = 0;
    double ke = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    Run<unsigned long long> run;
    unsigned long long *wsum = a.wsum + (int64_t)sp * g.ncell;

    for (int64_t grp = it.g0 + threadIdx.x; grp < it.g1; grp += blockDim.x) {
        const int64_t i0 = grp * PPT;
        double X[PPT], Y[PPT], Z[PPT], VX[PPT], VY[PPT], VZ[PPT];
        load_f64<PPT>(p.x, i0, X);
        load_f64<PPT>(p.y, i0, Y);
        load_f64<PPT>(p.z, i0, Z);
        if (kGather) {
            load_f64<PPT>(p.vx, i0, VX);
            load_f64<PPT>(p.vy, i0, VY);
            load_f64<PPT>(p.vz, i0, VZ);
        }
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            if (i0 + j >= end) continue;
            double x = X[j], y = Y[j], z = Z[j];
            if (kGather) {
                Split sx_, sy_, sz_;
                const int ix = split_cell(x, sx_), iy = split_cell(y, sy_), iz = split_cell(z, sz_);
                if ((unsigned)ix >= (unsigned)g.nx || (unsigned)iy >= (unsigned)g.ny ||
                    (unsigned)iz >= (unsigned)g.nz) {
                    flag_error(a.diag, OHPIC_ERR_BOUNDS, 1);
                    continue;
                }
                const int key = box.key(ix, iy, iz);
                nout += key < 0;
                d3 nd[8];
                load_nodes3(a, box, key, ix, iy, iz, sE, nd);
                double wx0, wx1, wy0, wy1, wz0, wz1;
                // x - floor(x) exactly (linear_interpolator.f90:47-52), from the bits
                cic<double>(a.weights, split_frac(sx_), wx0, wx1);
                cic<double>(a.weights, split_frac(sy_), wy0, wy1);
                cic<double>(a.weights, split_frac(sz_), wz0, wz1);
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
                                const d3 v = nd[ii + 2 * jj + 4 * kk];
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
                    // Strict: the half kick (qm*E)*dt2 in the reference's order.  Otherwise
                    // hq = qm*dt2 is rounded once on the host and each half kick is one
                    // FMA (six FP64 operations fewer per particle on the narrow FP64 pipe).
                    double upm0, upm1, upm2;
                    if (STRICT) {
                        const double qm = c.qm, dt2 = c.dt2;
                        upm0 = Ops::add(VX[j], Ops::mul(Ops::mul(qm, ex), dt2));
                        upm1 = Ops::add(VY[j], Ops::mul(Ops::mul(qm, ey), dt2));
                        upm2 = Ops::add(VZ[j], Ops::mul(Ops::mul(qm, ez), dt2));
                    } else {
                        upm0 = fma(c.hq, ex, VX[j]);
                        upm1 = fma(c.hq, ey, VY[j]);
                        upm2 = fma(c.hq, ez, VZ[j]);
                    }
                    const double upa0 = Ops::add(upm0, Ops::sub(Ops::mul(upm1, c.t[2]), Ops::mul(upm2, c.t[1])));
                    const double upa1 = Ops::add(upm1, Ops::sub(Ops::mul(upm2, c.t[0]), Ops::mul(upm0, c.t[2])));
                    const double upa2 = Ops::add(upm2, Ops::sub(Ops::mul(upm0, c.t[1]), Ops::mul(upm1, c.t[0])));
                    const double upp0 = Ops::add(upm0, Ops::sub(Ops::mul(upa1, c.s[2]), Ops::mul(upa2, c.s[1])));
                    const double upp1 = Ops::add(upm1, Ops::sub(Ops::mul(upa2, c.s[0]), Ops::mul(upa0, c.s[2])));
                    const double upp2 = Ops::add(upm2, Ops::sub(Ops::mul(upa0, c.s[1]), Ops::mul(upa1, c.s[0])));
                    if (STRICT) {
                        const double qm = c.qm, dt2 = c.dt2;
                        VX[j] = Ops::add(upp0, Ops::mul(Ops::mul(qm, ex), dt2));
                        VY[j] = Ops::add(upp1, Ops::mul(Ops::mul(qm, ey), dt2));
                        VZ[j] = Ops::add(upp2, Ops::mul(Ops::mul(qm, ez), dt2));
                    } else {
                        VX[j] = fma(c.hq, ex, upp0);
                        VY[j] = fma(c.hq, ey, upp1);
                        VZ[j] = fma(c.hq, ez, upp2);
                    }
                    // Position (:60-62) and the periodic boundary applied twice; the
                    // comparisons run on the bit patterns, the rare wraps in FP64.
                    x = Ops::add(x, Ops::mul(VX[j], c.dt));
                    y = Ops::add(y, Ops::mul(VY[j], c.dt));
                    z = Ops::add(z, Ops::mul(VZ[j], c.dt));
                    const bool wx = lt0(x) || ge_bits(x, bnx);
                    const bool wy = lt0(y) || ge_bits(y, bny);
                    const bool wz = lt0(z) || ge_bits(z, bnz);
                    ncx += wx; ncy += wy; ncz += wz;
                    if (wx || wy || wz) {
#pragma unroll
                        for (int rep = 0; rep < 2; ++rep) {
                            if (lt0(x)) x = Ops::add(fnx, x);
                            if (ge_bits(x, bnx)) x = Ops::sub(x, fnx);
                            if (lt0(y)) y = Ops::add(fny, y);
                            if (ge_bits(y, bny)) y = Ops::sub(y, fny);
                            if (lt0(z)) z = Ops::add(fnz, z);
                            if (ge_bits(z, bnz)) z = Ops::sub(z, fnz);
                        }
                    }
                    X[j] = x; Y[j] = y; Z[j] = z;
                    if (a.with_energy) {
                        ke = fma(VX[j], VX[j], fma(VY[j], VY[j], fma(VZ[j], VZ[j], ke)));
                        px += VX[j]; py += VY[j]; pz += VZ[j];
                    }
                }
            }
            if (kDeposit) {
                Split tx_, ty_, tz_;
                const int jx = split_cell(x, tx_), jy = split_cell(y, ty_), jz = split_cell(z, tz_);
                if ((unsigned)jx >= (unsigned)g.nx || (unsigned)jy >= (unsigned)g.ny ||
                    (unsigned)jz >= (unsigned)g.nz) {
                    flag_error(a.diag, OHPIC_ERR_BOUNDS, 2);
                    continue;
                }
                // rx*ry*rz of linear_scatter.f90:41-52 in 2^-48 fixed point; the
                // charge amount is applied per species when rho is formed
                unsigned long long w[8];
                fixed_weights48(a.weights, split_frac48(tx_), split_frac48(ty_), split_frac48(tz_), w);
                const int key = box.key(jx, jy, jz);
                if (key >= 0) {
                    run.add(key, w, sbox, box.sx, box.sxy);
                } else {
                    deposit_global48(g, wsum, jx, jy, jz, w, a.diag);
                    if (!kGather) ++nout;
                }
            }
        }
        if (kMove) {
            store_f64<PPT>(p.x, i0, X);
            store_f64<PPT>(p.y, i0, Y);
            store_f64<PPT>(p.z, i0, Z);
            store_f64<PPT>(p.vx, i0, VX);
            store_f64<PPT>(p.vy, i0, VY);
            store_f64<PPT>(p.vz, i0, VZ);
        }
    }
    if (kDeposit) run.flush(sbox, box.sx, box.sxy);
    if (kDeposit && box.on) {
        __syncthreads();
        flush_box48(a, it, sbox);
    }
    if (kMove || kGather) flush_diag<double>(a, sp, ncx, ncy, ncz, nout, ke, px, py, pz);
}

}  // namespace

template <typename P>
static void launch_k(ohpic_ctx *c, void (*kernel)(TileArgs, P), const TileArgs &a, int64_t blocks, size_t smem,
                     const P &parts)
{
    if (blocks <= 0) return;
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    kernel<<<(unsigned)blocks, 256, smem, c->stream>>>(a, parts);
    ++c->launches;
}

void launch_tiled_f64(ohpic_ctx *c, const TileArgs &a, int mode, int strict, int64_t blocks, size_t smem)
{
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
}

}  // namespace ohpic
