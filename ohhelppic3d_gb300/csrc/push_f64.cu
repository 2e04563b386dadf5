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
// extent, streams its particles with 16-byte vector loads and stores (2 FP64
// or 4 FP32 particles per thread per iteration) and flushes the rho box to
// global memory once.  A particle whose cell lies outside the staged box (it
// drifted since the last sort, or wrapped across the periodic edge) gathers
// from and deposits to global memory instead.
//
// Deposit.  A thread's consecutive particles are consecutive in cell order, so
// their CIC weights are summed in registers while they stay in one cell and the
// sum is added to the shared box with 8 shared atomics when the cell changes.
// Lanes of one warp that hit the same node serialise in the shared-memory unit
// only, which costs less than any warp-level reduction of 8 values.
#include "tile_common.cuh"

namespace ohpic {
namespace {

// ===========================================================================
// FP64 form: 2 particles per thread (double2 loads/stores).
// ===========================================================================
template <int MODE, bool STRICT>
__global__ void __launch_bounds__(256, 2) tiled_f64(TileArgs a, PartF64 p)
{
    constexpr int PPT = 2;
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
    double *srho = (double *)(smem + (kGather ? (size_t)s3 * sizeof(dnode) : 0));
    if (box.on) {
        stage_tile<dnode, double>(a, it, sE, srho, kGather, kDeposit);
        __syncthreads();
    }

    const int sp = it.sp;
    const SpeciesConst &c = a.sc[sp];
    const int64_t end = a.seg[sp] + a.count[sp];
    const double fnx = (double)g.nx, fny = (double)g.ny, fnz = (double)g.nz;
    const long long bnx = __double_as_longlong(fnx), bny = __double_as_longlong(fny), bnz = __double_as_longlong(fnz);
    unsigned ncx = 0, ncy = 0, ncz = 0, nout = 0;
    double ke = 0.0, px = 0.0, py = 0.0, pz = 0.0;
    Run<double> run;

    for (int64_t grp = it.g0 + threadIdx.x; grp < it.g1; grp += blockDim.x) {
        const int64_t i0 = grp * PPT;
        double X[PPT], Y[PPT], Z[PPT], VX[PPT], VY[PPT], VZ[PPT];
        {
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
#pragma unroll
        for (int j = 0; j < PPT; ++j) {
            if (i0 + j >= end) continue;
            double x = X[j], y = Y[j], z = Z[j];
            if (kGather) {
                const int ix = (int)x, iy = (int)y, iz = (int)z;
                if ((unsigned)ix >= (unsigned)g.nx || (unsigned)iy >= (unsigned)g.ny ||
                    (unsigned)iz >= (unsigned)g.nz) {
                    flag_error(a.diag, OHPIC_ERR_BOUNDS, 1);
                    continue;
                }
                const int key = box.key(ix, iy, iz);
                nout += key < 0;
                dnode nd[8];
                load_nodes<dnode>(a, box, key, ix, iy, iz, sE, nd);
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
                const double w[8] = {b00 * wz0, b10 * wz0, b01 * wz0, b11 * wz0,
                                     b00 * wz1, b10 * wz1, b01 * wz1, b11 * wz1};
                const int key = box.key(jx, jy, jz);
                if (key >= 0) {
                    run.add(key, w, srho, box.sx, box.sxy);
                } else {
                    deposit_global<double>(g, (double *)a.rho, jx, jy, jz, w);
                    if (!kGather) ++nout;
                }
            }
        }
        if (kMove) {
            *(double2 *)(p.x + i0) = make_double2(X[0], X[1]);
            *(double2 *)(p.y + i0) = make_double2(Y[0], Y[1]);
            *(double2 *)(p.z + i0) = make_double2(Z[0], Z[1]);
            *(double2 *)(p.vx + i0) = make_double2(VX[0], VX[1]);
            *(double2 *)(p.vy + i0) = make_double2(VY[0], VY[1]);
            *(double2 *)(p.vz + i0) = make_double2(VZ[0], VZ[1]);
        }
    }
    if (kDeposit) run.flush(srho, box.sx, box.sxy);
    if (kDeposit && box.on) {
        __syncthreads();
        flush_tile<double>(a, it, srho);
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
