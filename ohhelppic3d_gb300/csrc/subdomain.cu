// subdomain.cu -- one MPI rank's OhHelp subdomain, resident on its GPU (FP64 form).
//
// Reference path of a rank (src/ohhelppic3d.f90:286-381): scatter of the
// block's particles at local positions (linear_scatter.f90:22-55,
// ohfield.f90:199-206), the global field solve, interp + Boris + the periodic
// boundary twice (linear_interpolator.f90:33-67, particle_mover_boris.f90:37-62,
// periodic_particle_boundary.f90:42-53), correct_particle (ohhelp.f90:414-428)
// and transbound (ohhelp.f90:323-337).
//
// Layout.  The block's particles are SoA doubles (x, y, z, vx, vy, vz) plus an
// int64 pid, species s in slots [seg[s], seg[s] + cap[s]) of two buffers; the
// move's compaction writes the stayers into the other buffer in order.  Node
// fields cover the block's nodes lo .. lo + m (inclusive) on every axis: the
// per-species 2^-48 weight sums, rho, and E as three SoA blocks.
//
// The kernels are one particle per thread: a rank's subdomain is a share of the
// grid the tiled single-domain kernels serve, and this path exists for the
// integration, not for the single-GPU headline.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/ohpic_subdomain.h"
#include "f64_fixed.cuh"
#include "tile_common.cuh"

namespace ohpic {
namespace {

struct SubGeom {
    int n[3];        // global grid
    int lo[3];       // first cell of the block
    int m[3];        // cells of the block
    int sx;          // node pitches of the block arrays: m0 + 1, (m0 + 1)(m1 + 1)
    int64_t sxy;
    int64_t nodes;   // (m0 + 1)(m1 + 1)(m2 + 1)
};

struct SubPart {
    double *x, *y, *z, *vx, *vy, *vz;
    int64_t *pid;
};

__device__ __forceinline__ bool finite3(double x, double y, double z)
{
    return isfinite(x) && isfinite(y) && isfinite(z);
}

// Local cell of a global coordinate, or -1 outside the block.
__device__ __forceinline__ int local_cell(double x, int lo, int m, Split &s)
{
    const int c = split_cell(x, s) - lo;
    return (unsigned)c < (unsigned)m ? c : -1;
}

// Checks records before any is stored: species number, finite values, inside the block.
__global__ void k_sub_check(const ohpic_particle *in, int64_t n, int nspecies, SubGeom g, DevDiag *d)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const ohpic_particle r = in[i];
        const int s = r.spec - 1;
        if (s < 0 || s >= nspecies) {
            flag_error(d, OHPIC_ERR_INVALID, 30);
            continue;
        }
        if (!finite3(r.x, r.y, r.z) || !finite3(r.vx, r.vy, r.vz)) {
            flag_error(d, OHPIC_ERR_NONFINITE, 31);
            continue;
        }
        Split a, b, c;
        if (local_cell(r.x, g.lo[0], g.m[0], a) < 0 || local_cell(r.y, g.lo[1], g.m[1], b) < 0 ||
            local_cell(r.z, g.lo[2], g.m[2], c) < 0) {
            flag_error(d, OHPIC_ERR_BOUNDS, 32);
            continue;
        }
    }
}

// Records [0, n) of one species into slots dst .. dst + n (checked by k_sub_check).
__global__ void k_sub_store(const ohpic_particle *in, int64_t n, SubPart p, int64_t dst)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const ohpic_particle r = in[i];
        const int64_t o = dst + i;
        p.x[o] = r.x; p.y[o] = r.y; p.z[o] = r.z;
        p.vx[o] = r.vx; p.vy[o] = r.vy; p.vz[o] = r.vz;
        p.pid[o] = r.pid;
    }
}

__global__ void k_sub_fetch(SubPart p, int64_t src, int64_t n, int spec, ohpic_particle *out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = src + i;
        ohpic_particle r;
        r.x = p.x[o]; r.y = p.y[o]; r.z = p.z[o];
        r.vx = p.vx[o]; r.vy = p.vy[o]; r.vz = p.vz[o];
        r.pid = p.pid[o];
        r.nid = 13;
        r.spec = spec;
        out[i] = r;
    }
}

// CIC deposit of one species at local positions (linear_scatter.f90:32-53):
// the weights of the FP64 form's fixed-point deposit into the block's sums.
__global__ void k_sub_deposit(SubPart p, int64_t off, int64_t n, SubGeom g, int weights, unsigned long long *w,
                              DevDiag *d)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        Split a, b, c;
        const int lx = local_cell(p.x[off + i], g.lo[0], g.m[0], a);
        const int ly = local_cell(p.y[off + i], g.lo[1], g.m[1], b);
        const int lz = local_cell(p.z[off + i], g.lo[2], g.m[2], c);
        if ((lx | ly | lz) < 0) {
            flag_error(d, OHPIC_ERR_BOUNDS, 33);
            continue;
        }
        unsigned long long u[8];
        fixed_weights48(weights, split_frac48(a), split_frac48(b), split_frac48(c), u);
        unsigned long long *q = w + lx + (int64_t)g.sx * ly + g.sxy * lz;
        const int64_t off8[8] = {0, 1, g.sx, g.sx + 1, g.sxy, g.sxy + 1, g.sxy + g.sx, g.sxy + g.sx + 1};
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            const unsigned long long old = atomicAdd(q + off8[v], u[v]);
            if (old + u[v] < old) flag_error(d, OHPIC_ERR_CAPACITY, 34);
        }
    }
}

struct Charges {
    double q[OHPIC_MAX_SPECIES];
    int nspecies;
};

// rho = sum_s q_s W_s 2^-48 in species order, as the single-domain solve forms it.
__global__ void k_sub_rho(const unsigned long long *w, int64_t nodes, Charges sc, double *rho)
{
    constexpr double kUnit48 = 1.0 / 281474976710656.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nodes; t += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int s = 0; s < sc.nspecies; ++s) acc += sc.q[s] * (double)w[s * nodes + t];
        rho[t] = acc * kUnit48;
    }
}

// Side of the block a coordinate lies on: -1 below, +1 at or above the upper
// face, 0 inside (always 0 on an axis the block spans whole).
__device__ __forceinline__ int side(double x, int lo, int m, int n)
{
    if (m == n) return 0;
    if (x < (double)lo) return -1;
    return x >= (double)(lo + m) ? 1 : 0;
}

// One species: gather + Boris + position + periodic boundary twice, all in the
// reference's operation order (the strict arithmetic of the single-domain
// ohpic_move); then ownership: flag[i] = 1 when the new position has left the
// block, nid[i] the direction it left in (from the position before the wrap).
__global__ void k_sub_move(SubPart p, int64_t off, int64_t n, SubGeom g, const double *e, SpeciesConst c,
                           int weights, uint32_t *flag, int32_t *nid, DevDiag *d)
{
    using Ops = StrictOps;
    const double fn[3] = {(double)g.n[0], (double)g.n[1], (double)g.n[2]};
    const long long bn[3] = {__double_as_longlong(fn[0]), __double_as_longlong(fn[1]), __double_as_longlong(fn[2])};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = off + i;
        double x = p.x[o], y = p.y[o], z = p.z[o];
        Split a, b, cc;
        const int lx = local_cell(x, g.lo[0], g.m[0], a);
        const int ly = local_cell(y, g.lo[1], g.m[1], b);
        const int lz = local_cell(z, g.lo[2], g.m[2], cc);
        if ((lx | ly | lz) < 0) {
            flag_error(d, OHPIC_ERR_BOUNDS, 35);
            flag[i] = 0;
            nid[i] = 13;
            continue;
        }
        double wx0, wx1, wy0, wy1, wz0, wz1;
        cic<double>(weights, split_frac(a), wx0, wx1);
        cic<double>(weights, split_frac(b), wy0, wy1);
        cic<double>(weights, split_frac(cc), wz0, wz1);
        const double wxs[2] = {wx0, wx1}, wys[2] = {wy0, wy1}, wzs[2] = {wz0, wz1};
        // ret = ret + v*rx*ry*rz, i (x) outermost (linear_interpolator.f90:62-66)
        const int64_t base = lx + (int64_t)g.sx * ly + g.sxy * lz;
        double ex = 0.0, ey = 0.0, ez = 0.0;
#pragma unroll
        for (int ii = 0; ii < 2; ++ii)
#pragma unroll
            for (int jj = 0; jj < 2; ++jj)
#pragma unroll
                for (int kk = 0; kk < 2; ++kk) {
                    const int64_t q = base + ii + g.sx * jj + g.sxy * kk;
                    const double vx_ = __ldg(e + q), vy_ = __ldg(e + g.nodes + q), vz_ = __ldg(e + 2 * g.nodes + q);
                    ex = Ops::add(ex, Ops::mul(Ops::mul(Ops::mul(vx_, wxs[ii]), wys[jj]), wzs[kk]));
                    ey = Ops::add(ey, Ops::mul(Ops::mul(Ops::mul(vy_, wxs[ii]), wys[jj]), wzs[kk]));
                    ez = Ops::add(ez, Ops::mul(Ops::mul(Ops::mul(vz_, wxs[ii]), wys[jj]), wzs[kk]));
                }
        // Boris (particle_mover_boris.f90:42-56)
        const double qm = c.qm, dt2 = c.dt2;
        const double upm0 = Ops::add(p.vx[o], Ops::mul(Ops::mul(qm, ex), dt2));
        const double upm1 = Ops::add(p.vy[o], Ops::mul(Ops::mul(qm, ey), dt2));
        const double upm2 = Ops::add(p.vz[o], Ops::mul(Ops::mul(qm, ez), dt2));
        const double upa0 = Ops::add(upm0, Ops::sub(Ops::mul(upm1, c.t[2]), Ops::mul(upm2, c.t[1])));
        const double upa1 = Ops::add(upm1, Ops::sub(Ops::mul(upm2, c.t[0]), Ops::mul(upm0, c.t[2])));
        const double upa2 = Ops::add(upm2, Ops::sub(Ops::mul(upm0, c.t[1]), Ops::mul(upm1, c.t[0])));
        const double upp0 = Ops::add(upm0, Ops::sub(Ops::mul(upa1, c.s[2]), Ops::mul(upa2, c.s[1])));
        const double upp1 = Ops::add(upm1, Ops::sub(Ops::mul(upa2, c.s[0]), Ops::mul(upa0, c.s[2])));
        const double upp2 = Ops::add(upm2, Ops::sub(Ops::mul(upa0, c.s[1]), Ops::mul(upa1, c.s[0])));
        const double vx = Ops::add(upp0, Ops::mul(Ops::mul(qm, ex), dt2));
        const double vy = Ops::add(upp1, Ops::mul(Ops::mul(qm, ey), dt2));
        const double vz = Ops::add(upp2, Ops::mul(Ops::mul(qm, ez), dt2));
        // position (:60-62), then the side of the block before the periodic wrap
        x = Ops::add(x, Ops::mul(vx, c.dt));
        y = Ops::add(y, Ops::mul(vy, c.dt));
        z = Ops::add(z, Ops::mul(vz, c.dt));
        const int dx = side(x, g.lo[0], g.m[0], g.n[0]);
        const int dy = side(y, g.lo[1], g.m[1], g.n[1]);
        const int dz = side(z, g.lo[2], g.m[2], g.n[2]);
        // periodic_particle_boundary.f90:42-53, applied twice (ohhelppic3d.f90:353,355)
#pragma unroll
        for (int rep = 0; rep < 2; ++rep) {
            if (lt0(x)) x = Ops::add(fn[0], x);
            if (ge_bits(x, bn[0])) x = Ops::sub(x, fn[0]);
            if (lt0(y)) y = Ops::add(fn[1], y);
            if (ge_bits(y, bn[1])) y = Ops::sub(y, fn[1]);
            if (lt0(z)) z = Ops::add(fn[2], z);
            if (ge_bits(z, bn[2])) z = Ops::sub(z, fn[2]);
        }
        p.x[o] = x; p.y[o] = y; p.z[o] = z;
        p.vx[o] = vx; p.vy[o] = vy; p.vz[o] = vz;
        Split t;
        const bool home = local_cell(x, g.lo[0], g.m[0], t) >= 0 && local_cell(y, g.lo[1], g.m[1], t) >= 0 &&
                          local_cell(z, g.lo[2], g.m[2], t) >= 0;
        flag[i] = home ? 0u : 1u;
        nid[i] = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
    }
}

// Compaction after the move: stayer i to slot dst + i - ex[i] of the other
// buffer (order kept), emigrant i to out[ex[i]] (ex = exclusive scan of flag).
__global__ void k_sub_compact(SubPart src, SubPart dst, int64_t off, int64_t n, const uint32_t *flag,
                              const uint32_t *ex, const int32_t *nid, int spec, ohpic_particle *out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = off + i;
        if (flag[i]) {
            ohpic_particle r;
            r.x = src.x[o]; r.y = src.y[o]; r.z = src.z[o];
            r.vx = src.vx[o]; r.vy = src.vy[o]; r.vz = src.vz[o];
            r.pid = src.pid[o];
            r.nid = nid[i];
            r.spec = spec;
            out[ex[i]] = r;
        } else {
            const int64_t j = off + i - ex[i];
            dst.x[j] = src.x[o]; dst.y[j] = src.y[o]; dst.z[j] = src.z[o];
            dst.vx[j] = src.vx[o]; dst.vy[j] = src.vy[o]; dst.vz[j] = src.vz[o];
            dst.pid[j] = src.pid[o];
        }
    }
}

int grid_for(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return b < 1 ? 1 : (int)b;
}

}  // namespace
}  // namespace ohpic

using namespace ohpic;

struct ohpic_subdomain {
    int dev = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    ohpic_config cfg{};
    SubGeom g{};
    int nspecies = 0;
    int64_t cap[OHPIC_MAX_SPECIES] = {0}, seg[OHPIC_MAX_SPECIES] = {0}, count[OHPIC_MAX_SPECIES] = {0};
    int64_t total = 0, max_cap = 0;
    SpeciesConst sc[OHPIC_MAX_SPECIES];
    double sc_dt = -1.0;
    SubPart p[2]{};
    int cur = 0;
    void *block[2] = {nullptr, nullptr};
    unsigned long long *wsum = nullptr;
    double *rho = nullptr, *e = nullptr;
    uint32_t *flag = nullptr, *ex = nullptr, *scan_tmp = nullptr;
    int32_t *nid = nullptr;
    ohpic_particle *stage = nullptr;   // uploads, downloads and the emigrant box
    int64_t stage_cap = 0;
    int64_t emigrants = 0;             // records waiting at the front of the stage
    bool e_set = false;
    DevDiag *diag = nullptr;
};

namespace {

int sub_fail(ohpic_subdomain *sd, int code, const std::string &msg)
{
    if (sd) sd->err = msg;
    return code;
}

template <typename T>
int sub_alloc(ohpic_subdomain *sd, T **p, int64_t elems)
{
    *p = nullptr;
    const size_t bytes = sizeof(T) * (size_t)std::max<int64_t>(elems, 1);
    const cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return sub_fail(sd, OHPIC_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    return OHPIC_OK;
}

int sub_sync(ohpic_subdomain *sd)
{
    cudaError_t e = cudaStreamSynchronize(sd->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return sub_fail(sd, OHPIC_ERR_CUDA, std::string("subdomain: ") + cudaGetErrorString(e));
    int code[2] = {0, 0};
    cudaMemcpy(code, &sd->diag->err_code, 2 * sizeof(int), cudaMemcpyDeviceToHost);
    if (code[0] != 0) {
        cudaMemset(&sd->diag->err_code, 0, 2 * sizeof(int));
        return sub_fail(sd, code[0], "subdomain: device error flag " + std::to_string(code[0]) + " at site " +
                                         std::to_string(code[1]));
    }
    return OHPIC_OK;
}

}  // namespace

extern "C" {

int ohpic_sub_create(const ohpic_config *cfg, const int32_t lo[3], const int32_t m[3], ohpic_subdomain **out)
{
    if (!out) return OHPIC_ERR_INVALID;
    *out = nullptr;
    if (!cfg || !lo || !m) return OHPIC_ERR_INVALID;
    const int n[3] = {cfg->nx, cfg->ny, cfg->nz};
    for (int d = 0; d < 3; ++d)
        if (n[d] < 1 || m[d] < 1 || lo[d] < 0 || lo[d] + m[d] > n[d] || n[d] > (1 << 29)) return OHPIC_ERR_INVALID;
    if (cfg->precision != OHPIC_FP64 || cfg->nspecies < 1 || cfg->nspecies > OHPIC_MAX_SPECIES)
        return OHPIC_ERR_INVALID;
    ohpic_subdomain *sd = new ohpic_subdomain();
    sd->cfg = *cfg;
    sd->dev = cfg->device;
    sd->nspecies = cfg->nspecies;
    for (int d = 0; d < 3; ++d) {
        sd->g.n[d] = n[d];
        sd->g.lo[d] = lo[d];
        sd->g.m[d] = m[d];
    }
    sd->g.sx = m[0] + 1;
    sd->g.sxy = (int64_t)(m[0] + 1) * (m[1] + 1);
    sd->g.nodes = sd->g.sxy * (m[2] + 1);
    int64_t off = 0;
    for (int s = 0; s < sd->nspecies; ++s) {
        if (cfg->capacity[s] < 0) {
            delete sd;
            return OHPIC_ERR_INVALID;
        }
        sd->cap[s] = cfg->capacity[s];
        sd->seg[s] = off;
        off += (cfg->capacity[s] + 63) / 64 * 64;
        sd->max_cap = std::max(sd->max_cap, cfg->capacity[s]);
    }
    sd->total = std::max<int64_t>(off, 64);
    int rc = cudaSetDevice(sd->dev) == cudaSuccess ? OHPIC_OK : OHPIC_ERR_CUDA;
    if (rc == OHPIC_OK && cudaStreamCreateWithFlags(&sd->stream, cudaStreamNonBlocking) != cudaSuccess)
        rc = OHPIC_ERR_CUDA;
    const int64_t N = sd->total;
    for (int b = 0; b < 2 && rc == OHPIC_OK; ++b) {
        char *base = nullptr;
        rc = sub_alloc(sd, &base, 7 * 8 * N);
        if (rc != OHPIC_OK) break;
        sd->block[b] = base;
        double **arr[6] = {&sd->p[b].x, &sd->p[b].y, &sd->p[b].z, &sd->p[b].vx, &sd->p[b].vy, &sd->p[b].vz};
        for (int a = 0; a < 6; ++a) *arr[a] = (double *)(base + (size_t)a * 8 * N);
        sd->p[b].pid = (int64_t *)(base + (size_t)6 * 8 * N);
    }
    if (rc == OHPIC_OK) rc = sub_alloc(sd, &sd->wsum, (int64_t)sd->nspecies * sd->g.nodes);
    if (rc == OHPIC_OK) rc = sub_alloc(sd, &sd->rho, sd->g.nodes);
    if (rc == OHPIC_OK) rc = sub_alloc(sd, &sd->e, 3 * sd->g.nodes);
    if (rc == OHPIC_OK) rc = sub_alloc(sd, &sd->flag, std::max<int64_t>(sd->max_cap, 1));
    if (rc == OHPIC_OK) rc = sub_alloc(sd, &sd->ex, std::max<int64_t>(sd->max_cap, 1));
    if (rc == OHPIC_OK) rc = sub_alloc(sd, &sd->nid, std::max<int64_t>(sd->max_cap, 1));
    if (rc == OHPIC_OK) rc = sub_alloc(sd, &sd->scan_tmp, scan_tmp_elems(std::max<int64_t>(sd->max_cap, 1)));
    sd->stage_cap = std::max<int64_t>(N, 1);
    if (rc == OHPIC_OK) rc = sub_alloc(sd, &sd->stage, sd->stage_cap);
    if (rc == OHPIC_OK) rc = sub_alloc(sd, &sd->diag, 1);
    if (rc == OHPIC_OK && cudaMemset(sd->diag, 0, sizeof(DevDiag)) != cudaSuccess) rc = OHPIC_ERR_CUDA;
    if (rc == OHPIC_OK && cudaMemset(sd->e, 0, sizeof(double) * 3 * sd->g.nodes) != cudaSuccess) rc = OHPIC_ERR_CUDA;
    if (rc != OHPIC_OK) {
        ohpic_sub_destroy(sd);
        return rc;
    }
    *out = sd;
    return OHPIC_OK;
}

int ohpic_sub_destroy(ohpic_subdomain *sd)
{
    if (!sd) return OHPIC_OK;
    cudaSetDevice(sd->dev);
    if (sd->stream) cudaStreamSynchronize(sd->stream);
    void *ptrs[] = {sd->block[0], sd->block[1], sd->wsum, sd->rho, sd->e, sd->flag, sd->ex, sd->nid, sd->scan_tmp,
                    sd->stage, sd->diag};
    for (void *q : ptrs)
        if (q) cudaFree(q);
    if (sd->stream) cudaStreamDestroy(sd->stream);
    delete sd;
    return OHPIC_OK;
}

int ohpic_sub_append(ohpic_subdomain *sd, const ohpic_particle *p, int64_t n)
{
    if (!sd) return OHPIC_ERR_INVALID;
    if (n < 0 || (n > 0 && !p)) return sub_fail(sd, OHPIC_ERR_INVALID, "append: bad count or buffer");
    if (n == 0) return OHPIC_OK;
    cudaSetDevice(sd->dev);
    if (sd->emigrants > 0)
        return sub_fail(sd, OHPIC_ERR_INVALID, "append: take the emigrants of the last move first");
    // per-species counts on the host decide where each record goes
    int64_t add[OHPIC_MAX_SPECIES] = {0};
    for (int64_t i = 0; i < n; ++i) {
        const int s = p[i].spec - 1;
        if (s < 0 || s >= sd->nspecies) return sub_fail(sd, OHPIC_ERR_INVALID, "append: spec outside 1..nspecies");
        ++add[s];
    }
    for (int s = 0; s < sd->nspecies; ++s)
        if (sd->count[s] + add[s] > sd->cap[s])
            return sub_fail(sd, OHPIC_ERR_CAPACITY, "append: species " + std::to_string(s + 1) + " over capacity");
    if (n > sd->stage_cap) return sub_fail(sd, OHPIC_ERR_CAPACITY, "append: more records than the block holds");
    // validate every record on the device before any is stored
    if (cudaMemcpyAsync(sd->stage, p, sizeof(ohpic_particle) * (size_t)n, cudaMemcpyHostToDevice, sd->stream) !=
        cudaSuccess)
        return sub_fail(sd, OHPIC_ERR_CUDA, "append: copy failed");
    k_sub_check<<<grid_for(n), 256, 0, sd->stream>>>(sd->stage, n, sd->nspecies, sd->g, sd->diag);
    int rc = sub_sync(sd);
    if (rc != OHPIC_OK) return rc;
    // group by species on the host (records arrive mixed), one copy per species
    std::vector<ohpic_particle> by(n);
    int64_t start[OHPIC_MAX_SPECIES + 1] = {0};
    for (int s = 0; s < sd->nspecies; ++s) start[s + 1] = start[s] + add[s];
    int64_t fill[OHPIC_MAX_SPECIES];
    for (int s = 0; s < sd->nspecies; ++s) fill[s] = start[s];
    for (int64_t i = 0; i < n; ++i) by[fill[p[i].spec - 1]++] = p[i];
    if (cudaMemcpyAsync(sd->stage, by.data(), sizeof(ohpic_particle) * (size_t)n, cudaMemcpyHostToDevice,
                        sd->stream) != cudaSuccess)
        return sub_fail(sd, OHPIC_ERR_CUDA, "append: copy failed");
    for (int s = 0; s < sd->nspecies; ++s) {
        if (add[s] == 0) continue;
        k_sub_store<<<grid_for(add[s]), 256, 0, sd->stream>>>(sd->stage + start[s], add[s], sd->p[sd->cur],
                                                              sd->seg[s] + sd->count[s]);
        sd->count[s] += add[s];
    }
    return sub_sync(sd);
}

int ohpic_sub_count(ohpic_subdomain *sd, int species, int64_t *n)
{
    if (!sd || !n || species < 0 || species >= sd->nspecies) return OHPIC_ERR_INVALID;
    *n = sd->count[species];
    return OHPIC_OK;
}

int ohpic_sub_download(ohpic_subdomain *sd, int species, ohpic_particle *out, int64_t capacity, int64_t *n_out)
{
    if (!sd || species < 0 || species >= sd->nspecies) return OHPIC_ERR_INVALID;
    const int64_t n = sd->count[species];
    if (n_out) *n_out = n;
    if (n == 0) return OHPIC_OK;
    if (!out || capacity < n) return sub_fail(sd, OHPIC_ERR_CAPACITY, "download: buffer holds fewer records");
    if (sd->emigrants > 0) return sub_fail(sd, OHPIC_ERR_INVALID, "download: take the emigrants first");
    cudaSetDevice(sd->dev);
    k_sub_fetch<<<grid_for(n), 256, 0, sd->stream>>>(sd->p[sd->cur], sd->seg[species], n, species + 1, sd->stage);
    if (cudaMemcpyAsync(out, sd->stage, sizeof(ohpic_particle) * (size_t)n, cudaMemcpyDeviceToHost, sd->stream) !=
        cudaSuccess)
        return sub_fail(sd, OHPIC_ERR_CUDA, "download: copy failed");
    return sub_sync(sd);
}

int ohpic_sub_scatter(ohpic_subdomain *sd, double *rho)
{
    if (!sd || !rho) return OHPIC_ERR_INVALID;
    cudaSetDevice(sd->dev);
    const SubGeom &g = sd->g;
    cudaMemsetAsync(sd->wsum, 0, sizeof(unsigned long long) * (size_t)(sd->nspecies * g.nodes), sd->stream);
    for (int s = 0; s < sd->nspecies; ++s) {
        if (sd->count[s] == 0) continue;
        k_sub_deposit<<<grid_for(sd->count[s]), 256, 0, sd->stream>>>(sd->p[sd->cur], sd->seg[s], sd->count[s], g,
                                                                      sd->cfg.weights, sd->wsum + s * g.nodes,
                                                                      sd->diag);
    }
    Charges sc;
    sc.nspecies = sd->nspecies;
    for (int s = 0; s < OHPIC_MAX_SPECIES; ++s) sc.q[s] = s < sd->nspecies ? sd->cfg.q[s] : 0.0;
    k_sub_rho<<<grid_for(g.nodes), 256, 0, sd->stream>>>(sd->wsum, g.nodes, sc, sd->rho);
    if (cudaMemcpyAsync(rho, sd->rho, sizeof(double) * (size_t)g.nodes, cudaMemcpyDeviceToHost, sd->stream) !=
        cudaSuccess)
        return sub_fail(sd, OHPIC_ERR_CUDA, "scatter: copy failed");
    return sub_sync(sd);
}

int ohpic_sub_set_e(ohpic_subdomain *sd, const double *e)
{
    if (!sd || !e) return OHPIC_ERR_INVALID;
    cudaSetDevice(sd->dev);
    if (cudaMemcpyAsync(sd->e, e, sizeof(double) * 3 * (size_t)sd->g.nodes, cudaMemcpyHostToDevice, sd->stream) !=
        cudaSuccess)
        return sub_fail(sd, OHPIC_ERR_CUDA, "set_e: copy failed");
    sd->e_set = true;
    return sub_sync(sd);
}

int ohpic_sub_move(ohpic_subdomain *sd, double dt, int64_t *emigrants)
{
    if (!sd) return OHPIC_ERR_INVALID;
    if (!sd->e_set) return sub_fail(sd, OHPIC_ERR_INVALID, "move: no E block set");
    if (sd->emigrants > 0) return sub_fail(sd, OHPIC_ERR_INVALID, "move: take the emigrants of the last move first");
    cudaSetDevice(sd->dev);
    if (sd->sc_dt != dt) {
        for (int s = 0; s < sd->nspecies; ++s) species_consts(sd->cfg, s, dt, sd->sc[s]);
        sd->sc_dt = dt;
    }
    const int src = sd->cur, dst = 1 - sd->cur;
    int64_t left[OHPIC_MAX_SPECIES] = {0};
    int64_t out = 0;
    for (int s = 0; s < sd->nspecies; ++s) {
        const int64_t n = sd->count[s];
        if (n == 0) continue;
        k_sub_move<<<grid_for(n), 256, 0, sd->stream>>>(sd->p[src], sd->seg[s], n, sd->g, sd->e, sd->sc[s],
                                                        sd->cfg.weights, sd->flag, sd->nid, sd->diag);
        scan_u32(sd->stream, sd->flag, sd->ex, n, sd->scan_tmp);
        k_sub_compact<<<grid_for(n), 256, 0, sd->stream>>>(sd->p[src], sd->p[dst], sd->seg[s], n, sd->flag, sd->ex,
                                                           sd->nid, s + 1, sd->stage + out);
        uint32_t last[2] = {0, 0};
        cudaMemcpyAsync(&last[0], sd->ex + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, sd->stream);
        cudaMemcpyAsync(&last[1], sd->flag + n - 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, sd->stream);
        int rc = sub_sync(sd);
        if (rc != OHPIC_OK) return rc;
        left[s] = (int64_t)last[0] + last[1];
        out += left[s];
    }
    // species without particles keep their (empty) slots; the others moved to dst
    sd->cur = dst;
    for (int s = 0; s < sd->nspecies; ++s) {
        sd->count[s] -= left[s];
        if (emigrants) emigrants[s] = left[s];
    }
    sd->emigrants = out;
    return OHPIC_OK;
}

int ohpic_sub_take_emigrants(ohpic_subdomain *sd, ohpic_particle *out, int64_t capacity, int64_t *n_out)
{
    if (!sd) return OHPIC_ERR_INVALID;
    if (n_out) *n_out = sd->emigrants;
    if (sd->emigrants == 0 || (!out && capacity == 0)) return OHPIC_OK;   // nothing, or a query of the count
    if (!out || capacity < sd->emigrants) return sub_fail(sd, OHPIC_ERR_CAPACITY, "emigrants: buffer too small");
    cudaSetDevice(sd->dev);
    if (cudaMemcpyAsync(out, sd->stage, sizeof(ohpic_particle) * (size_t)sd->emigrants, cudaMemcpyDeviceToHost,
                        sd->stream) != cudaSuccess)
        return sub_fail(sd, OHPIC_ERR_CUDA, "emigrants: copy failed");
    const int rc = sub_sync(sd);
    if (rc == OHPIC_OK) sd->emigrants = 0;
    return rc;
}

int ohpic_sub_last_error(const ohpic_subdomain *sd, char *buf, size_t len)
{
    if (!buf || len == 0) return OHPIC_ERR_INVALID;
    const std::string &m = sd ? sd->err : std::string("null subdomain");
    const size_t k = std::min(len - 1, m.size());
    m.copy(buf, k);
    buf[k] = 0;
    return OHPIC_OK;
}

}  // extern "C"
