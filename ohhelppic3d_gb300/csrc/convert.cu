// convert.cu -- conversions between the host FP64 particle records and the
// device forms, kinetic-energy reduction, and the dispatch of the tiled kernels.
#include <cuda_runtime.h>
#include <stdint.h>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ void flag_error(DevDiag *d, int code, int info)
{
    if (atomicCAS(&d->err_code, 0, code) == 0) d->err_info = info;
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
    if (!isfinite(x)) {   // floor(NaN) converts to cell 0 with a NaN offset: refuse it
        flag_error(d, OHPIC_ERR_NONFINITE, 12);
        i = 0;
        o = 0.f;
        return;
    }
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

// The FP32 push trusts its particles (no per-particle checks), so an upload
// refuses velocities that are not finite in FP32.
__device__ __forceinline__ void check_velocity(double vx, double vy, double vz, DevDiag *d)
{
    if (!(isfinite((float)vx) && isfinite((float)vy) && isfinite((float)vz))) flag_error(d, OHPIC_ERR_NONFINITE, 13);
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
        check_velocity(r[3], r[4], r[5], d);
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

// Direct forms: the six FP64 arrays are the caller's host arrays, read or written
// by the kernel itself.  Pinned host memory is reachable from the GPU at the same
// address (over NVLink-C2C on Grace), so no device staging copy is needed.
__global__ void k_soa_to_f32(Soa6 s, int64_t n, PartF32 p, uint32_t *ids, int64_t dst, uint32_t id0, int nx, int ny,
                             int nz, DevDiag *d)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int ix, iy, iz;
        float ox, oy, oz;
        split_pos(s.p[0][i], nx, ix, ox, d);
        split_pos(s.p[1][i], ny, iy, oy, d);
        split_pos(s.p[2][i], nz, iz, oz, d);
        const int64_t o = dst + i;
        p.cell[o] = pack_cell(ix, iy, iz);
        p.ox[o] = ox; p.oy[o] = oy; p.oz[o] = oz;
        const double vx = s.p[3][i], vy = s.p[4][i], vz = s.p[5][i];
        p.vx[o] = (float)vx; p.vy[o] = (float)vy; p.vz[o] = (float)vz;
        check_velocity(vx, vy, vz, d);
        if (ids) ids[o] = id0 + (uint32_t)i;
    }
}

__global__ void k_soa_to_f64(Soa6 s, int64_t n, PartF64 p, uint32_t *ids, int64_t dst, uint32_t id0)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = dst + i;
        p.x[o] = s.p[0][i]; p.y[o] = s.p[1][i]; p.z[o] = s.p[2][i];
        p.vx[o] = s.p[3][i]; p.vy[o] = s.p[4][i]; p.vz[o] = s.p[5][i];
        if (ids) ids[o] = id0 + (uint32_t)i;
    }
}

__global__ void k_f32_to_soa(PartF32 p, int64_t src, int64_t n, Soa6w out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = src + i;
        const int32_t c = p.cell[o];
        if (out.p[0]) out.p[0][i] = (double)cell_x(c) + (double)p.ox[o];
        if (out.p[1]) out.p[1][i] = (double)cell_y(c) + (double)p.oy[o];
        if (out.p[2]) out.p[2][i] = (double)cell_z(c) + (double)p.oz[o];
        if (out.p[3]) out.p[3][i] = p.vx[o];
        if (out.p[4]) out.p[4][i] = p.vy[o];
        if (out.p[5]) out.p[5][i] = p.vz[o];
    }
}

__global__ void k_f64_to_soa(PartF64 p, int64_t src, int64_t n, Soa6w out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = src + i;
        if (out.p[0]) out.p[0][i] = p.x[o];
        if (out.p[1]) out.p[1][i] = p.y[o];
        if (out.p[2]) out.p[2][i] = p.z[o];
        if (out.p[3]) out.p[3][i] = p.vx[o];
        if (out.p[4]) out.p[4][i] = p.vy[o];
        if (out.p[5]) out.p[5][i] = p.vz[o];
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
void launch_tiled(ohpic_ctx *c, int mode, int strict)
{
    TileArgs a;
    a.g = c->g;
    a.nspecies = c->cfg.nspecies;
    a.weights = c->cfg.weights;
    a.split = c->split;
    a.deposit = c->dep_strategy;
    if (c->sorted && mode != MODE_DEPOSIT) ensure_emap(c);
    a.use_tma = c->sorted && c->emap_ok ? 1 : 0;
    a.with_energy = c->with_energy ? 1 : 0;
    a.sorted = c->sorted ? 1 : 0;
    a.ppl = c->cfg.precision == OHPIC_FP32 && (mode == MODE_PUSH || mode == MODE_DEPOSIT) ? c->lane_particles : 2;
    a.tma_polls = c->tma_polls;
    a.chunk = 4096;
    for (int s = 0; s < OHPIC_MAX_SPECIES; ++s) {
        a.seg[s] = c->seg[s];
        a.count[s] = c->count[s];
        a.sc[s] = c->sc[s];
    }
    a.tile_begin = c->tile_begin;
    a.epad = c->epad;
    a.rho = c->rho;
    a.wsum = c->wsum;
    a.interp_out = c->interp_buf;
    a.diag = c->diag;

    const bool f64 = c->cfg.precision == OHPIC_FP64;
    // particles per thread per iteration: 2 in both forms (double2 / float2 vectors)
    const int PPT = 2;
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
    // E box: 4 reals per node; deposit box: one real per node (FP64) or the
    // low and high 32-bit words of the fixed-point sums (FP32).
    // (+128: the kernels align the box start to 128 bytes for TMA)
    if (a.sorted) smem = (gather ? s3 * 4 * es : 0) + (dep ? s3 * 8 : 0) + 128;
    // four per lane (FP32 push/deposit): the boxes end on a 16-byte boundary and are
    // followed by the per-thread prefetch stage (7 arrays x 256 threads x 16 bytes)
    if (!f64 && a.ppl == 4) smem = (a.sorted ? ((s3 * 4 * es + s3 * 8 + 15) & ~(size_t)15) : 0) + kQuadStageBytes + 128;
    if (f64) {
        launch_tiled_f64(c, a, mode, strict, blocks, smem);
        return;
    }
    // The push right after a sort reads the sort's records when it runs the
    // default shape (four per lane, LANES deposit, tiles); anything else needs
    // the word arrays first.
    const bool from_rec = c->rec_pending && mode == MODE_PUSH && a.sorted && a.ppl == 4 &&
                          a.deposit == OHPIC_DEPOSIT_LANES;
    if (!from_rec) {
        materialize_records(c);
        launch_tiled_f32(c, a, mode, blocks, smem);
        return;
    }
    const RecIn rin{(const int4 *)c->pblock[1 - c->cur], c->ids[c->cur]};
    launch_tiled_f32(c, a, mode, blocks, smem, &rin);
    c->rec_pending = false;
}

void launch_f64_soa_from_stage(ohpic_ctx *c, const double *stage, int64_t n, int64_t dst, uint32_t id0, int aos,
                               int64_t stride_doubles)
{
    materialize_records(c);
    if (n <= 0) return;
    k_stage_to_f64<<<grid_for(n, 256), 256, 0, c->stream>>>(stage, n, aos, stride_doubles, c->p64[c->cur],
                                                             c->ids[c->cur], dst, id0);
    ++c->launches;
}

void launch_f64_to_f32(ohpic_ctx *c, const double *stage, int64_t n, int64_t dst, uint32_t id0, int aos,
                       int64_t stride_doubles)
{
    materialize_records(c);
    if (n <= 0) return;
    k_stage_to_f32<<<grid_for(n, 256), 256, 0, c->stream>>>(stage, n, aos, stride_doubles, c->p32[c->cur],
                                                             c->ids[c->cur], dst, id0, c->g.nx, c->g.ny,
                                                             c->g.nz, c->diag);
    ++c->launches;
}

void launch_from_host_soa(ohpic_ctx *c, const Soa6 &s, int64_t n, int64_t dst, uint32_t id0)
{
    materialize_records(c);
    if (n <= 0) return;
    if (c->cfg.precision == OHPIC_FP64)
        k_soa_to_f64<<<grid_for(n, 256), 256, 0, c->stream>>>(s, n, c->p64[c->cur], c->ids[c->cur], dst, id0);
    else
        k_soa_to_f32<<<grid_for(n, 256), 256, 0, c->stream>>>(s, n, c->p32[c->cur], c->ids[c->cur], dst, id0, c->g.nx,
                                                               c->g.ny, c->g.nz, c->diag);
    ++c->launches;
}

void launch_to_host_soa(ohpic_ctx *c, const Soa6w &out, int64_t src, int64_t n)
{
    materialize_records(c);
    if (n <= 0) return;
    if (c->cfg.precision == OHPIC_FP64)
        k_f64_to_soa<<<grid_for(n, 256), 256, 0, c->stream>>>(c->p64[c->cur], src, n, out);
    else
        k_f32_to_soa<<<grid_for(n, 256), 256, 0, c->stream>>>(c->p32[c->cur], src, n, out);
    ++c->launches;
}

void launch_to_f64_stage(ohpic_ctx *c, double *stage, int64_t src, int64_t n)
{
    materialize_records(c);
    if (n <= 0) return;
    if (c->cfg.precision == OHPIC_FP64)
        k_f64_to_stage<<<grid_for(n, 256), 256, 0, c->stream>>>(c->p64[c->cur], src, n, stage);
    else
        k_f32_to_stage<<<grid_for(n, 256), 256, 0, c->stream>>>(c->p32[c->cur], src, n, stage);
    ++c->launches;
}

void launch_kinetic(ohpic_ctx *c)
{
    materialize_records(c);
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
