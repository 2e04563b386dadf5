// ohpic_api.cu -- the extern "C" entry points declared in include/ohpic.h.
//
// The context replaces the state the reference keeps in module variables of
// src/ohhelppic3d.f90:1-58 (parameters, fields eb/rho/phi, particle buffer,
// scatter, interpolator, mover, boundaries, field solver).  Every entry point
// checks its arguments, enqueues work on the context's stream and returns a
// status; nothing throws across the ABI.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>

#include "ohpic_internal.cuh"
#include "tma.cuh"

using namespace ohpic;

namespace {

int fail(ohpic_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

int64_t align_up(int64_t v, int64_t a) { return (v + a - 1) / a * a; }

// Largest power-of-two tile edge <= 8 that divides n.
int default_tile(int n)
{
    for (int t = 8; t > 1; t >>= 1)
        if (n % t == 0) return t;
    return 1;
}

}  // namespace

namespace ohpic {

// Grid geometry for a tile shape and halo; false when a tile edge is not a
// divisor of the grid or the staged box does not fit one CTA's shared memory.
bool make_geom(const ohpic_config &k, const int tile[3], int halo, Geom &g)
{
    const int n[3] = {k.nx, k.ny, k.nz};
    for (int d = 0; d < 3; ++d)
        if (tile[d] < 1 || tile[d] > 64 || n[d] % tile[d] != 0) return false;
    if (halo < 0 || halo > kMaxHalo) return false;
    g.nx = k.nx; g.ny = k.ny; g.nz = k.nz;
    g.tx = tile[0]; g.ty = tile[1]; g.tz = tile[2];
    g.ntx = g.nx / g.tx; g.nty = g.ny / g.ty; g.ntz = g.nz / g.tz;
    g.halo = halo;
    g.sx = g.tx + 2 * halo + 1; g.sy = g.ty + 2 * halo + 1; g.sz = g.tz + 2 * halo + 1;
    g.gx = g.nx + 2 * halo + 1; g.gy = g.ny + 2 * halo + 1; g.gz = g.nz + 2 * halo + 1;
    g.ncell = (int64_t)g.nx * g.ny * g.nz;
    g.ntile = (int64_t)g.ntx * g.nty * g.ntz;
    g.tile_cells = g.tx * g.ty * g.tz;
    g.nxh = g.nx / 2 + 1;
    g.nspec = (int64_t)g.nxh * g.ny * g.nz;
    // Staged E box (4 reals per node) plus the deposit box (8 bytes per node).
    const int64_t s3 = (int64_t)g.sx * g.sy * g.sz;
    const int64_t es = k.precision == OHPIC_FP64 ? 8 : 4;
    // (leaves room for the FP32 push's 28 KB prefetch stage within a CTA's 227 KB)
    return s3 * (4 * es + 8) <= 192 * 1024;
}

// Boris constants of one species for a time step (particle_mover_boris.f90:37-43),
// evaluated in FP64 in the reference's operation order (host code is built
// with -ffp-contract=off).
void species_consts(const ohpic_config &cfg, int s, double dt, SpeciesConst &k)
{
    k.qm = cfg.qm[s];
    k.q = cfg.q[s];
    k.dt = dt;
    k.dt2 = dt * 0.5;
    for (int d = 0; d < 3; ++d) k.t[d] = k.qm * cfg.b0[d] * k.dt2;
    const double tt = k.t[0] * k.t[0] + k.t[1] * k.t[1] + k.t[2] * k.t[2];
    for (int d = 0; d < 3; ++d) k.s[d] = 2.0 * k.t[d] / (1.0 + tt);
    k.mass = k.q / k.qm;
    k.hq = k.qm * k.dt2;
    k.hq32 = (float)k.hq;
    k.dt32 = (float)dt;
    for (int d = 0; d < 3; ++d) {
        k.t32[d] = (float)k.t[d];
        k.s32[d] = (float)k.s[d];
    }
}

// The device address of a host array the GPU can reach directly (pinned with
// cudaHostAlloc/cudaMallocHost or registered with cudaHostRegister), else null.
const void *device_view(const void *host)
{
    if (!host) return nullptr;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

}  // namespace ohpic

namespace {

void set_dt(ohpic_ctx *c, double dt)
{
    if (c->sc_dt == dt) return;
    for (int s = 0; s < c->cfg.nspecies; ++s) species_consts(c->cfg, s, dt, c->sc[s]);
    c->sc_dt = dt;
}

template <typename T>
int dalloc(ohpic_ctx *c, T **p, int64_t elems)
{
    *p = nullptr;
    if (elems <= 0) elems = 1;
    const size_t bytes = sizeof(T) * (size_t)elems;
    cudaError_t e = cudaMalloc((void **)p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(c, OHPIC_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                                          cudaGetErrorString(e));
    }
    c->device_bytes += (int64_t)bytes;
    return OHPIC_OK;
}

void dfree(void *p)
{
    if (p) cudaFree(p);
}

// Device error flag raised by a kernel (bounds), read after a synchronise.
int check_device(ohpic_ctx *c)
{
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return fail(c, OHPIC_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(e));
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, OHPIC_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    int code = 0, info = 0;
    cudaMemcpy(&code, &c->diag->err_code, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemcpy(&info, &c->diag->err_info, sizeof(int), cudaMemcpyDeviceToHost);
    if (code != 0) {
        cudaMemset(&c->diag->err_code, 0, 2 * sizeof(int));
        return fail(c, code, "device error flag " + std::to_string(code) + " at site " + std::to_string(info));
    }
    return OHPIC_OK;
}

bool species_ok(const ohpic_ctx *c, int s) { return c && s >= 0 && s < c->cfg.nspecies; }

// An upload the conversion kernel flagged (a position it cannot wrap, a
// non-finite value) leaves the species empty, so no kernel reads the bad particle.
int check_upload(ohpic_ctx *c, int s)
{
    const int rc = check_device(c);
    if (rc != OHPIC_OK) c->count[s] = 0;
    return rc;
}

// Clears the deposit target: the per-species fixed-point weight sums (units of
// 2^-24 in the FP32 form, 2^-48 in the FP64 form), turned into rho by the next
// solve or download.
void zero_deposit(ohpic_ctx *c)
{
    launch_zero(c, c->wsum, (int64_t)c->cfg.nspecies * c->g.ncell * 8);
    c->rho_from_wsum = true;
}

int do_scatter(ohpic_ctx *c)
{
    zero_deposit(c);
    launch_tiled(c, MODE_DEPOSIT, 0);
    c->rho_valid = true;
    return OHPIC_OK;
}

int do_solve(ohpic_ctx *c)
{
    if (!c->rho_valid) do_scatter(c);
    const int rc = solve_fields(c);
    if (rc == OHPIC_OK) c->field_valid = true;
    return rc;
}

int do_push(ohpic_ctx *c, double dt)
{
    set_dt(c, dt);
    // crossings + outside (+ the kinetic sums when the push tracks them)
    cudaMemsetAsync(c->diag, 0, c->with_energy ? offsetof(DevDiag, charge) : offsetof(DevDiag, kin), c->stream);
    c->kin_valid = c->with_energy;
    zero_deposit(c);
    if (c->push_timing) {
        // One event pair per push kernel, summed by ohpic_stats.
        const size_t need = 2 * (size_t)(c->ev_used + 1);
        while (c->ev_pool.size() < need) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) break;
            c->ev_pool.push_back(e);
        }
        if (c->ev_pool.size() >= need) {
            cudaEventRecord(c->ev_pool[2 * c->ev_used], c->stream);
            launch_tiled(c, MODE_PUSH, 0);
            cudaEventRecord(c->ev_pool[2 * c->ev_used + 1], c->stream);
            ++c->ev_used;
            ++c->push_launches;
        } else {
            launch_tiled(c, MODE_PUSH, 0);
        }
    } else {
        launch_tiled(c, MODE_PUSH, 0);
    }
    c->rho_valid = true;
    c->field_valid = false;
    ++c->steps;
    ++c->steps_since_sort;
    return OHPIC_OK;
}

// ---- checkpoint / restart: snapshot byte image ----
const char kSnapMagic[8] = {'O', 'H', 'P', 'I', 'C', 'S', 'N', '1'};

struct SnapHeader {
    char magic[8];
    int32_t version, precision, nx, ny, nz, nspecies, track_ids, reserved;
    int64_t steps, steps_since_sort;
    int64_t count[OHPIC_MAX_SPECIES];
    char pad[256 - 8 - 8 * 4 - 2 * 8 - 8 * OHPIC_MAX_SPECIES];
};
static_assert(sizeof(SnapHeader) == 256, "snapshot header is 256 bytes");

// A restored FP32 snapshot must hold what the push relies on without checking:
// cells inside the grid, offsets in [0, 1) and finite velocities.  Species
// segment from index `seg`, n particles.
__global__ void k_check_restored(PartF32 p, int64_t seg, int64_t n, int nx, int ny, int nz, DevDiag *d)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = seg + i;
        const int32_t c = p.cell[k];
        const float ox = p.ox[k], oy = p.oy[k], oz = p.oz[k];
        int code = 0, info = 0;
        if (cell_x(c) >= nx || cell_y(c) >= ny || cell_z(c) >= nz) {
            code = OHPIC_ERR_BOUNDS;
            info = 11;
        } else if (!(ox >= 0.f && ox < 1.f && oy >= 0.f && oy < 1.f && oz >= 0.f && oz < 1.f)) {
            code = isfinite(ox) && isfinite(oy) && isfinite(oz) ? OHPIC_ERR_BOUNDS : OHPIC_ERR_NONFINITE;
            info = 14;
        } else if (!(isfinite(p.vx[k]) && isfinite(p.vy[k]) && isfinite(p.vz[k]))) {
            code = OHPIC_ERR_NONFINITE;
            info = 15;
        }
        if (code && atomicCAS(&d->err_code, 0, code) == 0) d->err_info = info;
    }
}

// Bytes of one species' arrays: FP32 7 words + id; FP64 6 doubles + id, padded to 8.

int64_t snap_species_bytes(bool f64, int64_t n)
{
    return f64 ? (52 * n + 7) / 8 * 8 : 32 * n;
}

// The species' device arrays in snapshot order (byte addresses of element seg)
// and their element sizes; returns the count.
int snap_arrays(ohpic_ctx *c, int s, char *arr[7], int64_t es[7])
{
    materialize_records(c);
    const int64_t seg = c->seg[s];
    if (c->cfg.precision == OHPIC_FP64) {
        const PartF64 &q = c->p64[c->cur];
        double *a[6] = {q.x, q.y, q.z, q.vx, q.vy, q.vz};
        for (int k = 0; k < 6; ++k) {
            arr[k] = (char *)(a[k] + seg);
            es[k] = 8;
        }
        return 6;
    }
    const PartF32 &q = c->p32[c->cur];
    arr[0] = (char *)(q.cell + seg);
    es[0] = 4;
    float *a[6] = {q.ox, q.oy, q.oz, q.vx, q.vy, q.vz};
    for (int k = 0; k < 6; ++k) {
        arr[k + 1] = (char *)(a[k] + seg);
        es[k + 1] = 4;
    }
    return 7;
}

}  // namespace

extern "C" {

void ohpic_config_default(ohpic_config *cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->precision = OHPIC_FP64;
    cfg->weights = OHPIC_WEIGHTS_REFERENCE;
    cfg->sort_every = 20;
    cfg->track_ids = 1;
    cfg->device = 0;
}

const char *ohpic_status_string(int status)
{
    switch (status) {
    case OHPIC_OK: return "ok";
    case OHPIC_ERR_INVALID: return "invalid argument or configuration";
    case OHPIC_ERR_OOM: return "out of memory";
    case OHPIC_ERR_CUDA: return "CUDA error";
    case OHPIC_ERR_BOUNDS: return "index out of bounds on the device";
    case OHPIC_ERR_TIMEOUT: return "bounded device wait timed out";
    case OHPIC_ERR_CAPACITY: return "species capacity exceeded";
    case OHPIC_ERR_UNSUPPORTED: return "per-particle entry point not supported on the GPU";
    case OHPIC_ERR_NONFINITE: return "non-finite particle state";
    case OHPIC_ERR_REJECTED: return "request rejected";
    default: return "unknown status";
    }
}

int ohpic_destroy(ohpic_ctx *c)
{
    if (!c) return OHPIC_OK;
    cudaSetDevice(c->dev);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (int b = 0; b < 2; ++b) {
        dfree(c->pblock[b]);   // holds the particle arrays and the ids
    }
    dfree(c->rho); dfree(c->phi); dfree(c->epad); dfree(c->spec); dfree(c->green); dfree(c->wsum);
    dfree(c->cell_count); dfree(c->cell_stay); dfree(c->cell_start); dfree(c->scan_tmp); dfree(c->key_table); dfree(c->tile_begin);
    dfree(c->stage); dfree(c->interp_buf); dfree(c->diag);
    if (c->diag_host) cudaFreeHost(c->diag_host);
    fields_teardown(c);
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return OHPIC_OK;
}

int ohpic_create(const ohpic_config *cfg, ohpic_ctx **out)
{
    if (!cfg || !out) return OHPIC_ERR_INVALID;
    *out = nullptr;
    const ohpic_config &k = *cfg;
    if (k.nx < 1 || k.ny < 1 || k.nz < 1 || k.nspecies < 1 || k.nspecies > OHPIC_MAX_SPECIES)
        return OHPIC_ERR_INVALID;
    if (k.precision != OHPIC_FP64 && k.precision != OHPIC_FP32) return OHPIC_ERR_INVALID;
    if (k.weights != OHPIC_WEIGHTS_REFERENCE && k.weights != OHPIC_WEIGHTS_STANDARD) return OHPIC_ERR_INVALID;
    if (k.precision == OHPIC_FP32 && (k.nx > kMaxNx || k.ny > kMaxNy || k.nz > kMaxNz)) return OHPIC_ERR_INVALID;
    if ((int64_t)k.nx * k.ny * k.nz > (int64_t)1 << 31) return OHPIC_ERR_INVALID;
    for (int s = 0; s < k.nspecies; ++s) {
        if (k.capacity[s] < 0 || k.capacity[s] > (int64_t)UINT32_MAX) return OHPIC_ERR_INVALID;
        if (!(k.qm[s] != 0.0) || !std::isfinite(k.qm[s]) || !std::isfinite(k.q[s])) return OHPIC_ERR_INVALID;
    }
    const int tile[3] = {k.tile[0] > 0 ? k.tile[0] : default_tile(k.nx), k.tile[1] > 0 ? k.tile[1] : default_tile(k.ny),
                         k.tile[2] > 0 ? k.tile[2] : default_tile(k.nz)};
    const int n[3] = {k.nx, k.ny, k.nz};
    for (int d = 0; d < 3; ++d)
        if (n[d] % tile[d] != 0 || tile[d] > 64) return OHPIC_ERR_INVALID;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || k.device < 0 || k.device >= ndev) {
        cudaGetLastError();
        return OHPIC_ERR_CUDA;
    }
    ohpic_ctx *c = new (std::nothrow) ohpic_ctx();
    if (!c) return OHPIC_ERR_OOM;
    c->cfg = k;
    c->dev = k.device;
    cudaSetDevice(c->dev);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return OHPIC_ERR_CUDA;
    }

    c->halo = 2;
    c->split = 1;
    c->with_energy = false;
    c->sc_dt = NAN;
    c->dep_strategy = OHPIC_DEPOSIT_LANES;
    c->lane_particles = 4;
    c->sort_lead = 0;
    c->tma_polls = kTmaWaitPolls;
    Geom &g = c->g;
    if (!make_geom(k, tile, c->halo, g)) {
        ohpic_destroy(c);
        return OHPIC_ERR_INVALID;
    }

    int64_t off = 0;
    for (int s = 0; s < k.nspecies; ++s) {
        c->seg[s] = off;
        c->cap[s] = k.capacity[s];
        off = align_up(off + k.capacity[s], kSegAlign);
    }
    c->total_slots = std::max<int64_t>(off, kSegAlign);
    set_dt(c, k.dt);

    const bool f64 = k.precision == OHPIC_FP64;
    const int64_t es = f64 ? 8 : 4;
    int rc = OHPIC_OK;
    const int64_t N = c->total_slots;
    for (int b = 0; b < 2 && rc == OHPIC_OK; ++b) {
        // eight arrays of N elements of the form's width in one block (N sort records)
        const int64_t part = align_up(N * es, 256);
        rc = dalloc(c, (char **)&c->pblock[b], 8 * part);
        if (rc != OHPIC_OK) break;
        char *base = (char *)c->pblock[b];
        if (f64) {
            double **arr[6] = {&c->p64[b].x, &c->p64[b].y, &c->p64[b].z, &c->p64[b].vx, &c->p64[b].vy, &c->p64[b].vz};
            for (int a = 0; a < 6; ++a) *arr[a] = (double *)(base + a * part);
            if (k.track_ids) c->ids[b] = (uint32_t *)(base + 6 * part);
        } else {
            c->p32[b].cell = (int32_t *)base;
            float **arr[6] = {&c->p32[b].ox, &c->p32[b].oy, &c->p32[b].oz, &c->p32[b].vx, &c->p32[b].vy, &c->p32[b].vz};
            for (int a = 0; a < 6; ++a) *arr[a] = (float *)(base + (a + 1) * part);
            if (k.track_ids) c->ids[b] = (uint32_t *)(base + 7 * part);
        }
    }
    if (rc == OHPIC_OK) rc = dalloc(c, (char **)&c->rho, g.ncell * es);
    if (rc == OHPIC_OK) rc = dalloc(c, &c->wsum, (int64_t)k.nspecies * g.ncell);
    if (rc == OHPIC_OK) rc = dalloc(c, (char **)&c->phi, g.ncell * es);
    if (rc == OHPIC_OK) rc = dalloc(c, (char **)&c->epad, (int64_t)g.gx * g.gy * g.gz * 4 * es);
    if (rc == OHPIC_OK) rc = dalloc(c, (char **)&c->spec, g.nspec * 2 * es);
    if (rc == OHPIC_OK) rc = dalloc(c, &c->green, g.nspec);
    if (rc == OHPIC_OK) rc = dalloc(c, &c->cell_count, g.ncell);
    if (rc == OHPIC_OK) rc = dalloc(c, &c->cell_stay, g.ncell);
    if (rc == OHPIC_OK) rc = dalloc(c, &c->cell_start, g.ncell + 1);
    if (rc == OHPIC_OK) rc = dalloc(c, &c->scan_tmp, scan_tmp_elems(g.ncell));
    if (rc == OHPIC_OK) rc = dalloc(c, &c->key_table, (int64_t)g.nx + g.ny + g.nz);
    if (rc == OHPIC_OK) rc = dalloc(c, &c->tile_begin, (int64_t)k.nspecies * (g.ntile + 1));
    if (rc == OHPIC_OK) {
        // Staging: chunks of up to 4M particles (6 doubles) and 3 full fields.
        c->stage_bytes = std::max<int64_t>((int64_t)48 << 22, 3 * g.ncell * 8);
        c->stage_bytes = std::min<int64_t>(c->stage_bytes, std::max<int64_t>(48 * N + 4096, 3 * g.ncell * 8 + 4096));
        rc = dalloc(c, (char **)&c->stage, c->stage_bytes);
    }
    if (rc == OHPIC_OK) rc = dalloc(c, &c->diag, 1);
    if (rc == OHPIC_OK && cudaMallocHost((void **)&c->diag_host, sizeof(DevDiag)) != cudaSuccess)
        rc = fail(c, OHPIC_ERR_OOM, "pinned diag allocation failed");
    if (rc != OHPIC_OK) {
        std::string msg = c->err;
        ohpic_destroy(c);
        (void)msg;
        return rc;
    }
    cudaMemsetAsync(c->diag, 0, sizeof(DevDiag), c->stream);
    cudaMemsetAsync(c->epad, 0, (size_t)g.gx * g.gy * g.gz * 4 * es, c->stream);
    cudaMemsetAsync(c->rho, 0, (size_t)(g.ncell * es), c->stream);
    rc = fields_setup(c);
    if (rc == OHPIC_OK) rc = check_device(c);
    if (rc != OHPIC_OK) {
        ohpic_destroy(c);
        return rc;
    }
    *out = c;
    return OHPIC_OK;
}

int ohpic_upload_particles_soa(ohpic_ctx *c, int s, const double *x, const double *y, const double *z,
                               const double *vx, const double *vy, const double *vz, int64_t n)
{
    if (!species_ok(c, s) || n < 0) return fail(c, OHPIC_ERR_INVALID, "upload: bad species or count");
    if (n > c->cap[s]) return fail(c, OHPIC_ERR_CAPACITY, "upload: " + std::to_string(n) + " > capacity");
    if (n > 0 && (!x || !y || !z || !vx || !vy || !vz)) return fail(c, OHPIC_ERR_INVALID, "upload: null array");
    cudaSetDevice(c->dev);
    materialize_records(c);
    const int64_t chunk = std::max<int64_t>(1, c->stage_bytes / 48);
    double *stage = (double *)c->stage;
    const double *src[6] = {x, y, z, vx, vy, vz};
    // Arrays the GPU can reach (pinned or registered) are read by the conversion
    // kernel itself; others go through the device staging buffer chunk by chunk.
    Soa6 direct;
    bool all_direct = n > 0;
    for (int k = 0; k < 6 && all_direct; ++k) {
        direct.p[k] = (const double *)device_view(src[k]);
        all_direct = direct.p[k] != nullptr;
    }
    if (all_direct) launch_from_host_soa(c, direct, n, c->seg[s], 0);
    for (int64_t a = 0; a < n && !all_direct; a += chunk) {
        const int64_t m = std::min(chunk, n - a);
        for (int k = 0; k < 6; ++k)
            OHPIC_CUDA_TRY(c, cudaMemcpyAsync(stage + k * m, src[k] + a, sizeof(double) * m, cudaMemcpyHostToDevice,
                                              c->stream));
        if (c->cfg.precision == OHPIC_FP64)
            launch_f64_soa_from_stage(c, stage, m, c->seg[s] + a, (uint32_t)a, 0, 0);
        else
            launch_f64_to_f32(c, stage, m, c->seg[s] + a, (uint32_t)a, 0, 0);
        // The next chunk's copy into the stage is ordered after this conversion by the stream.
    }
    c->count[s] = n;
    c->sorted = false;
    c->rho_valid = false;
    c->kin_valid = false;
    return check_upload(c, s);
}

int ohpic_upload_particles(ohpic_ctx *c, int s, const void *pbuf, int64_t n, int64_t stride)
{
    if (!species_ok(c, s) || n < 0) return fail(c, OHPIC_ERR_INVALID, "upload: bad species or count");
    if (stride < 48 || stride % 8 != 0) return fail(c, OHPIC_ERR_INVALID, "upload: stride must be >= 48 and a multiple of 8");
    if (n > c->cap[s]) return fail(c, OHPIC_ERR_CAPACITY, "upload: " + std::to_string(n) + " > capacity");
    if (n > 0 && !pbuf) return fail(c, OHPIC_ERR_INVALID, "upload: null buffer");
    cudaSetDevice(c->dev);
    materialize_records(c);
    const int64_t chunk = std::max<int64_t>(1, c->stage_bytes / stride);
    for (int64_t a = 0; a < n; a += chunk) {
        const int64_t m = std::min(chunk, n - a);
        OHPIC_CUDA_TRY(c, cudaMemcpyAsync(c->stage, (const char *)pbuf + a * stride, (size_t)(m * stride),
                                          cudaMemcpyHostToDevice, c->stream));
        if (c->cfg.precision == OHPIC_FP64)
            launch_f64_soa_from_stage(c, (const double *)c->stage, m, c->seg[s] + a, (uint32_t)a, 1, stride / 8);
        else
            launch_f64_to_f32(c, (const double *)c->stage, m, c->seg[s] + a, (uint32_t)a, 1, stride / 8);
    }
    c->count[s] = n;
    c->sorted = false;
    c->rho_valid = false;
    c->kin_valid = false;
    return check_upload(c, s);
}

int ohpic_init_particles(ohpic_ctx *c, uint64_t initstate, uint64_t initseq, uint64_t advance,
                         const ohpic_species_init *species, int64_t *counts_out)
{
    if (!c || !species) return fail(c, OHPIC_ERR_INVALID, "init: null argument");
    for (int s = 0; s < c->cfg.nspecies; ++s) {
        const ohpic_species_init &p = species[s];
        if (!(p.ppc >= 0.0) || !std::isfinite(p.ppc) || !(p.vth >= 0.0) || !std::isfinite(p.vth))
            return fail(c, OHPIC_ERR_INVALID, "init: ppc and vth must be finite and >= 0");
    }
    cudaSetDevice(c->dev);
    materialize_records(c);
    const int rc = init_particles(c, initstate, initseq, advance, species, counts_out);
    if (rc != OHPIC_OK) return rc;
    return check_device(c);
}

int ohpic_download_particles_soa(ohpic_ctx *c, int s, double *x, double *y, double *z, double *vx, double *vy,
                                 double *vz, uint32_t *ids, int64_t capacity, int64_t *n_out)
{
    if (!species_ok(c, s)) return fail(c, OHPIC_ERR_INVALID, "download: bad species");
    const int64_t n = c->count[s];
    if (n_out) *n_out = n;
    if (capacity < n) return fail(c, OHPIC_ERR_CAPACITY, "download: host capacity too small");
    if (ids && !c->cfg.track_ids) return fail(c, OHPIC_ERR_INVALID, "download: ids requested but not tracked");
    cudaSetDevice(c->dev);
    materialize_records(c);
    const int64_t chunk = std::max<int64_t>(1, c->stage_bytes / 48);
    double *stage = (double *)c->stage;
    double *dst[6] = {x, y, z, vx, vy, vz};
    // Arrays the GPU can reach (pinned or registered) are written by the
    // conversion kernel itself; others come back through the staging buffer.
    Soa6w direct;
    bool all_direct = n > 0;
    for (int k = 0; k < 6 && all_direct; ++k) {
        direct.p[k] = dst[k] ? (double *)device_view(dst[k]) : nullptr;
        all_direct = !dst[k] || direct.p[k] != nullptr;
    }
    if (all_direct) {
        launch_to_host_soa(c, direct, c->seg[s], n);
        if (ids)
            OHPIC_CUDA_TRY(c, cudaMemcpyAsync(ids, c->ids[c->cur] + c->seg[s], sizeof(uint32_t) * n,
                                              cudaMemcpyDeviceToHost, c->stream));
    }
    for (int64_t a = 0; a < n && !all_direct; a += chunk) {
        const int64_t m = std::min(chunk, n - a);
        launch_to_f64_stage(c, stage, c->seg[s] + a, m);
        for (int k = 0; k < 6; ++k)
            if (dst[k])
                OHPIC_CUDA_TRY(c, cudaMemcpyAsync(dst[k] + a, stage + k * m, sizeof(double) * m,
                                                  cudaMemcpyDeviceToHost, c->stream));
        if (ids)
            OHPIC_CUDA_TRY(c, cudaMemcpyAsync(ids + a, c->ids[c->cur] + c->seg[s] + a, sizeof(uint32_t) * m,
                                              cudaMemcpyDeviceToHost, c->stream));
    }
    return check_device(c);
}

int ohpic_download_particles(ohpic_ctx *c, int s, void *pbuf, int64_t capacity, int64_t stride, int64_t *n_out)
{
    if (!species_ok(c, s)) return fail(c, OHPIC_ERR_INVALID, "download: bad species");
    if (stride < 48 || stride % 8 != 0) return fail(c, OHPIC_ERR_INVALID, "download: bad stride");
    const int64_t n = c->count[s];
    if (n_out) *n_out = n;
    if (capacity < n) return fail(c, OHPIC_ERR_CAPACITY, "download: host capacity too small");
    cudaSetDevice(c->dev);
    materialize_records(c);
    const int64_t chunk = std::max<int64_t>(1, c->stage_bytes / 48);
    double *stage = (double *)c->stage;
    for (int64_t a = 0; a < n; a += chunk) {
        const int64_t m = std::min(chunk, n - a);
        launch_to_f64_stage(c, stage, c->seg[s] + a, m);
        // Strided host writes: one 2-D copy per component.
        for (int k = 0; k < 6; ++k)
            OHPIC_CUDA_TRY(c, cudaMemcpy2DAsync((char *)pbuf + a * stride + 8 * k, (size_t)stride, stage + k * m,
                                                sizeof(double), sizeof(double), (size_t)m, cudaMemcpyDeviceToHost,
                                                c->stream));
    }
    return check_device(c);
}

int ohpic_scatter(ohpic_ctx *c)
{
    if (!c) return OHPIC_ERR_INVALID;
    cudaSetDevice(c->dev);
    return do_scatter(c);
}

int ohpic_solve(ohpic_ctx *c)
{
    if (!c) return OHPIC_ERR_INVALID;
    cudaSetDevice(c->dev);
    return do_solve(c);
}

int ohpic_interp(ohpic_ctx *c, int s, double *e_out, int64_t capacity, int64_t *n_out)
{
    if (!species_ok(c, s)) return fail(c, OHPIC_ERR_INVALID, "interp: bad species");
    const int64_t n = c->count[s];
    if (n_out) *n_out = n;
    if (capacity < 3 * n) return fail(c, OHPIC_ERR_CAPACITY, "interp: output capacity must be >= 3*count");
    cudaSetDevice(c->dev);
    if (!c->field_valid) {
        const int rc = do_solve(c);
        if (rc != OHPIC_OK) return rc;
    }
    // One slot of 3 doubles per particle slot of every species (absolute index).
    const int64_t need = 3 * c->total_slots;
    if (need > c->interp_cap) {
        dfree(c->interp_buf);
        c->interp_buf = nullptr;
        c->interp_cap = 0;
        const int rc = dalloc(c, &c->interp_buf, need);
        if (rc != OHPIC_OK) return rc;
        c->interp_cap = need;
    }
    const int strict = 1;
    launch_tiled(c, MODE_INTERP, strict);
    if (n > 0)
        OHPIC_CUDA_TRY(c, cudaMemcpyAsync(e_out, c->interp_buf + 3 * c->seg[s], sizeof(double) * 3 * n,
                                          cudaMemcpyDeviceToHost, c->stream));
    return check_device(c);
}

int ohpic_move(ohpic_ctx *c, double dt)
{
    if (!c || !std::isfinite(dt)) return fail(c, OHPIC_ERR_INVALID, "move: bad dt");
    cudaSetDevice(c->dev);
    if (!c->field_valid) {
        const int rc = do_solve(c);
        if (rc != OHPIC_OK) return rc;
    }
    set_dt(c, dt);
    cudaMemsetAsync(c->diag, 0, offsetof(DevDiag, kin), c->stream);
    launch_tiled(c, MODE_MOVE, c->cfg.precision == OHPIC_FP64 ? 1 : 0);
    c->rho_valid = false;
    c->field_valid = false;
    c->kin_valid = false;
    return OHPIC_OK;
}

int ohpic_push(ohpic_ctx *c, double dt)
{
    if (!c || !std::isfinite(dt)) return fail(c, OHPIC_ERR_INVALID, "push: bad dt");
    cudaSetDevice(c->dev);
    if (!c->field_valid) {
        const int rc = do_solve(c);
        if (rc != OHPIC_OK) return rc;
    }
    return do_push(c, dt);
}

int ohpic_sort(ohpic_ctx *c)
{
    if (!c) return OHPIC_ERR_INVALID;
    cudaSetDevice(c->dev);
    return sort_particles(c);
}

int ohpic_step(ohpic_ctx *c, double dt, int nsteps)
{
    if (!c || !std::isfinite(dt) || nsteps < 0) return fail(c, OHPIC_ERR_INVALID, "step: bad arguments");
    cudaSetDevice(c->dev);
    if (!c->sorted && c->cfg.sort_every > 0) {
        const int rc = sort_particles(c);
        if (rc != OHPIC_OK) return rc;
    }
    for (int i = 0; i < nsteps; ++i) {
        int rc = do_solve(c);
        if (rc == OHPIC_OK) rc = do_push(c, dt);
        if (rc == OHPIC_OK && c->cfg.sort_every > 0 && c->steps_since_sort >= c->cfg.sort_every)
            rc = sort_particles(c);
        if (rc != OHPIC_OK) return rc;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(c, OHPIC_ERR_CUDA, std::string("step: ") + cudaGetErrorString(e));
    return OHPIC_OK;
}

int ohpic_download_field(ohpic_ctx *c, int which, double *host)
{
    if (!c || which < OHPIC_RHO || which > OHPIC_EZ || !host) return fail(c, OHPIC_ERR_INVALID, "download_field: bad args");
    cudaSetDevice(c->dev);
    double *stage = (double *)c->stage;
    field_to_double(c, which, stage);
    OHPIC_CUDA_TRY(c, cudaMemcpyAsync(host, stage, sizeof(double) * c->g.ncell, cudaMemcpyDeviceToHost, c->stream));
    return check_device(c);
}

int ohpic_upload_field(ohpic_ctx *c, int which, const double *host)
{
    if (!c || which < OHPIC_RHO || which > OHPIC_EZ || !host) return fail(c, OHPIC_ERR_INVALID, "upload_field: bad args");
    cudaSetDevice(c->dev);
    double *stage = (double *)c->stage;
    OHPIC_CUDA_TRY(c, cudaMemcpyAsync(stage, host, sizeof(double) * c->g.ncell, cudaMemcpyHostToDevice, c->stream));
    field_from_double(c, which, stage);
    if (which == OHPIC_RHO) {
        c->rho_valid = true;
        c->rho_from_wsum = false;   // rho itself is now the charge density
        c->field_valid = false;
    } else if (which >= OHPIC_EX) {
        c->field_valid = true;
    }
    return check_device(c);
}

int ohpic_download_field_ohfield(ohpic_ctx *c, int which, double *values, int nelem, const int32_t lo[3],
                                 const int32_t hi[3])
{
    if (!c || !values || !lo || !hi) return fail(c, OHPIC_ERR_INVALID, "ohfield: null argument");
    if (which != OHPIC_RHO && which != OHPIC_PHI && which != OHPIC_EX)
        return fail(c, OHPIC_ERR_INVALID, "ohfield: which must be RHO, PHI or EX (eb)");
    const int need = which == OHPIC_EX ? 6 : 1;
    if (nelem < need) return fail(c, OHPIC_ERR_INVALID, "ohfield: nelem too small");
    for (int d = 0; d < 3; ++d)
        if (hi[d] < lo[d]) return fail(c, OHPIC_ERR_INVALID, "ohfield: empty range");
    const int ncomp = which == OHPIC_EX ? 3 : 1;
    const int64_t nc = c->g.ncell;
    double *tmp = nullptr;
    if (cudaMallocHost((void **)&tmp, sizeof(double) * nc * ncomp) != cudaSuccess)
        return fail(c, OHPIC_ERR_OOM, "ohfield: pinned buffer");
    int rc = OHPIC_OK;
    for (int k = 0; k < ncomp && rc == OHPIC_OK; ++k)
        rc = ohpic_download_field(c, which == OHPIC_EX ? OHPIC_EX + k : which, tmp + k * nc);
    if (rc == OHPIC_OK) {
        const int n[3] = {c->g.nx, c->g.ny, c->g.nz};
        const int64_t ex = hi[0] - lo[0] + 1, ey = hi[1] - lo[1] + 1;
        for (int z = lo[2]; z <= hi[2]; ++z)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int x = lo[0]; x <= hi[0]; ++x) {
                    const int i = ((x % n[0]) + n[0]) % n[0], j = ((y % n[1]) + n[1]) % n[1],
                              kk = ((z % n[2]) + n[2]) % n[2];
                    const int64_t src = i + (int64_t)n[0] * (j + (int64_t)n[1] * kk);
                    double *dst = values + (int64_t)nelem * ((x - lo[0]) + ex * ((y - lo[1]) + ey * (int64_t)(z - lo[2])));
                    for (int k = 0; k < ncomp; ++k) dst[k] = tmp[k * nc + src];
                    if (which == OHPIC_EX)
                        for (int k = 0; k < 3; ++k) dst[3 + k] = c->cfg.b0[k];
                }
    }
    cudaFreeHost(tmp);
    return rc;
}

int ohpic_diagnostics(ohpic_ctx *c, ohpic_diag *d)
{
    if (!c || !d) return OHPIC_ERR_INVALID;
    cudaSetDevice(c->dev);
    if (!c->rho_valid) do_scatter(c);
    launch_field_energy(c);
    if (!c->kin_valid) launch_kinetic(c);
    OHPIC_CUDA_TRY(c, cudaMemcpyAsync(c->diag_host, c->diag, sizeof(DevDiag), cudaMemcpyDeviceToHost, c->stream));
    const int rc = check_device(c);
    if (rc != OHPIC_OK) return rc;
    const DevDiag &h = *c->diag_host;
    memset(d, 0, sizeof(*d));
    for (int s = 0; s < c->cfg.nspecies; ++s) {
        d->count[s] = c->count[s];
        const double m = c->cfg.q[s] / c->cfg.qm[s];
        d->kinetic_energy += 0.5 * m * h.kin[s][0];
        for (int k = 0; k < 3; ++k) d->momentum[k] += m * h.kin[s][1 + k];
    }
    for (int k = 0; k < 3; ++k) d->crossings[k] = (int64_t)h.crossings[k];
    d->outside_tile = (int64_t)h.outside;
    d->step = c->steps;
    d->total_charge = h.charge;
    d->field_energy = h.field_energy;
    return OHPIC_OK;
}

int ohpic_set_energy_tracking(ohpic_ctx *c, int enable)
{
    if (!c) return OHPIC_ERR_INVALID;
    c->with_energy = enable != 0;
    c->kin_valid = false;
    return OHPIC_OK;
}

int ohpic_set_tma_wait_limit(ohpic_ctx *c, uint32_t polls)
{
    if (!c) return OHPIC_ERR_INVALID;
    c->tma_polls = polls;
    return OHPIC_OK;
}

int ohpic_move_one(ohpic_ctx *c, double *, double, const double *, double)
{
    return fail(c, OHPIC_ERR_UNSUPPORTED, "per-particle move is not served from device memory; use ohpic_move");
}

int ohpic_scatter_one(ohpic_ctx *c, const double *, double, int)
{
    return fail(c, OHPIC_ERR_UNSUPPORTED, "per-particle scatter is not served from device memory; use ohpic_scatter");
}

int ohpic_last_error(const ohpic_ctx *c, char *buf, size_t len)
{
    if (!c || !buf || len == 0) return OHPIC_ERR_INVALID;
    const size_t n = std::min(len - 1, c->err.size());
    memcpy(buf, c->err.data(), n);
    buf[n] = 0;
    return OHPIC_OK;
}

int ohpic_synchronize(ohpic_ctx *c)
{
    if (!c) return OHPIC_ERR_INVALID;
    cudaSetDevice(c->dev);
    return check_device(c);
}

int ohpic_get_stream(ohpic_ctx *c, void **stream)
{
    if (!c || !stream) return OHPIC_ERR_INVALID;
    *stream = (void *)c->stream;
    return OHPIC_OK;
}

int ohpic_set_push_timing(ohpic_ctx *c, int enable)
{
    if (!c) return OHPIC_ERR_INVALID;
    c->push_timing = enable != 0;
    c->push_ms = 0.0;
    c->push_launches = 0;
    return OHPIC_OK;
}

int ohpic_stats(ohpic_ctx *c, int64_t *launches, int64_t *push_launches, double *push_ms)
{
    if (!c) return OHPIC_ERR_INVALID;
    if (c->ev_used > 0) {
        cudaSetDevice(c->dev);
        OHPIC_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        for (int i = 0; i < c->ev_used; ++i) {
            float ms = 0.f;
            OHPIC_CUDA_TRY(c, cudaEventElapsedTime(&ms, c->ev_pool[2 * i], c->ev_pool[2 * i + 1]));
            c->push_ms += ms;
        }
        c->ev_used = 0;
    }
    if (launches) *launches = c->launches;
    if (push_launches) *push_launches = c->push_launches;
    if (push_ms) *push_ms = c->push_ms;
    return OHPIC_OK;
}

int ohpic_memory(ohpic_ctx *c, int64_t *bytes)
{
    if (!c || !bytes) return OHPIC_ERR_INVALID;
    *bytes = c->device_bytes;
    return OHPIC_OK;
}

int ohpic_get_tuning(ohpic_ctx *c, ohpic_tuning *t)
{
    if (!c || !t) return OHPIC_ERR_INVALID;
    t->tile[0] = c->g.tx;
    t->tile[1] = c->g.ty;
    t->tile[2] = c->g.tz;
    t->halo = c->g.halo;
    t->split = c->split;
    t->deposit = c->dep_strategy;
    t->lane_particles = c->lane_particles;
    t->sort_every = c->cfg.sort_every;
    t->sort_lead = c->sort_lead;
    return OHPIC_OK;
}

int ohpic_set_tuning(ohpic_ctx *c, const ohpic_tuning *t)
{
    if (!c || !t) return OHPIC_ERR_INVALID;
    if (t->split < 1 || t->split > 64 || t->deposit < OHPIC_DEPOSIT_RUNS || t->deposit > OHPIC_DEPOSIT_LANES ||
        t->sort_every < 0 || (t->lane_particles != 2 && t->lane_particles != 4))
        return fail(c, OHPIC_ERR_INVALID,
                    "tuning: split 1..64, deposit 0..4, sort_every >= 0, lane_particles 2 or 4");
    if (t->sort_lead < 0 || t->sort_lead > 4096 || (t->sort_lead != 0 && c->cfg.precision != OHPIC_FP32))
        return fail(c, OHPIC_ERR_INVALID, "tuning: sort_lead 0..4096, nonzero only in the FP32 form");
    Geom g2;
    if (!make_geom(c->cfg, t->tile, t->halo, g2))
        return fail(c, OHPIC_ERR_INVALID, "tuning: tile edges must divide the grid (<= 64) and the staged box fit");
    cudaSetDevice(c->dev);
    materialize_records(c);
    const bool relayout = g2.tx != c->g.tx || g2.ty != c->g.ty || g2.tz != c->g.tz || g2.halo != c->g.halo;
    if (relayout) {
        OHPIC_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
        const int64_t es = c->cfg.precision == OHPIC_FP64 ? 8 : 4;
        if (g2.halo != c->g.halo) {
            dfree(c->epad);
            c->device_bytes -= (int64_t)c->g.gx * c->g.gy * c->g.gz * 4 * es;
            int rc = dalloc(c, (char **)&c->epad, (int64_t)g2.gx * g2.gy * g2.gz * 4 * es);
            if (rc != OHPIC_OK) return rc;
            cudaMemsetAsync(c->epad, 0, (size_t)g2.gx * g2.gy * g2.gz * 4 * es, c->stream);
        }
        if (g2.ntile != c->g.ntile) {
            dfree(c->tile_begin);
            c->device_bytes -= (int64_t)c->cfg.nspecies * (c->g.ntile + 1) * 8;
            int rc = dalloc(c, &c->tile_begin, (int64_t)c->cfg.nspecies * (g2.ntile + 1));
            if (rc != OHPIC_OK) return rc;
        }
        c->g = g2;
        c->halo = g2.halo;
        c->cfg.tile[0] = g2.tx;
        c->cfg.tile[1] = g2.ty;
        c->cfg.tile[2] = g2.tz;
        c->sorted = false;
        c->field_valid = false;
    }
    c->split = t->split;
    c->dep_strategy = t->deposit;
    c->lane_particles = t->lane_particles;
    c->cfg.sort_every = t->sort_every;
    c->sort_lead = t->sort_lead;
    return OHPIC_OK;
}

int ohpic_snapshot_size(ohpic_ctx *c, int64_t *bytes)
{
    if (!c || !bytes) return fail(c, OHPIC_ERR_INVALID, "snapshot_size: null argument");
    const bool f64 = c->cfg.precision == OHPIC_FP64;
    int64_t b = (int64_t)sizeof(SnapHeader);
    for (int s = 0; s < c->cfg.nspecies; ++s) b += snap_species_bytes(f64, c->count[s]);
    *bytes = b;
    return OHPIC_OK;
}

int ohpic_snapshot_save(ohpic_ctx *c, void *host, int64_t bytes)
{
    if (!c || !host) return fail(c, OHPIC_ERR_INVALID, "snapshot_save: null argument");
    int64_t need = 0;
    ohpic_snapshot_size(c, &need);
    if (bytes < need) return fail(c, OHPIC_ERR_CAPACITY, "snapshot_save: buffer smaller than ohpic_snapshot_size");
    cudaSetDevice(c->dev);
    materialize_records(c);
    const bool f64 = c->cfg.precision == OHPIC_FP64;
    SnapHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kSnapMagic, sizeof(h.magic));
    h.version = 1;
    h.precision = c->cfg.precision;
    h.nx = c->cfg.nx; h.ny = c->cfg.ny; h.nz = c->cfg.nz;
    h.nspecies = c->cfg.nspecies;
    h.track_ids = c->cfg.track_ids ? 1 : 0;
    h.steps = c->steps;
    h.steps_since_sort = c->steps_since_sort;
    for (int s = 0; s < c->cfg.nspecies; ++s) h.count[s] = c->count[s];
    memcpy(host, &h, sizeof(h));
    char *p = (char *)host + sizeof(h);
    for (int s = 0; s < c->cfg.nspecies; ++s) {
        const int64_t n = c->count[s];
        const int64_t sb = snap_species_bytes(f64, n);
        char *arr[7];
        int64_t es[7];
        const int na = snap_arrays(c, s, arr, es);
        memset(p, 0, (size_t)sb);   // ids when not tracked, and the FP64 padding
        int64_t off = 0;
        for (int k = 0; k < na && n > 0; ++k) {
            OHPIC_CUDA_TRY(c, cudaMemcpyAsync(p + off, arr[k], (size_t)(es[k] * n), cudaMemcpyDeviceToHost, c->stream));
            off += es[k] * n;
        }
        if (n > 0 && c->ids[c->cur])
            OHPIC_CUDA_TRY(c, cudaMemcpyAsync(p + off, c->ids[c->cur] + c->seg[s], sizeof(uint32_t) * n,
                                              cudaMemcpyDeviceToHost, c->stream));
        p += sb;
    }
    OHPIC_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    return check_device(c);
}

int ohpic_snapshot_load(ohpic_ctx *c, const void *host, int64_t bytes)
{
    if (!c || !host) return fail(c, OHPIC_ERR_INVALID, "snapshot_load: null argument");
    if (bytes < (int64_t)sizeof(SnapHeader)) return fail(c, OHPIC_ERR_INVALID, "snapshot_load: truncated snapshot");
    SnapHeader h;
    memcpy(&h, host, sizeof(h));
    if (memcmp(h.magic, kSnapMagic, sizeof(h.magic)) != 0 || h.version != 1)
        return fail(c, OHPIC_ERR_INVALID, "snapshot_load: not an ohpic snapshot (magic or version)");
    if (h.precision != c->cfg.precision || h.nx != c->cfg.nx || h.ny != c->cfg.ny || h.nz != c->cfg.nz ||
        h.nspecies != c->cfg.nspecies)
        return fail(c, OHPIC_ERR_INVALID, "snapshot_load: grid, precision form or species count differ");
    if (c->cfg.track_ids && !h.track_ids)
        return fail(c, OHPIC_ERR_INVALID, "snapshot_load: the context tracks ids but the snapshot has none");
    const bool f64 = c->cfg.precision == OHPIC_FP64;
    int64_t need = (int64_t)sizeof(SnapHeader);
    for (int s = 0; s < h.nspecies; ++s) {
        if (h.count[s] < 0 || h.count[s] > c->cap[s])
            return fail(c, OHPIC_ERR_CAPACITY, "snapshot_load: species " + std::to_string(s) + " count " +
                                                   std::to_string(h.count[s]) + " exceeds the capacity");
        need += snap_species_bytes(f64, h.count[s]);
    }
    if (bytes < need) return fail(c, OHPIC_ERR_INVALID, "snapshot_load: truncated snapshot");
    cudaSetDevice(c->dev);
    materialize_records(c);
    const char *p = (const char *)host + sizeof(h);
    for (int s = 0; s < h.nspecies; ++s) {
        const int64_t n = h.count[s];
        char *arr[7];
        int64_t es[7];
        const int na = snap_arrays(c, s, arr, es);
        int64_t off = 0;
        for (int k = 0; k < na && n > 0; ++k) {
            OHPIC_CUDA_TRY(c, cudaMemcpyAsync(arr[k], p + off, (size_t)(es[k] * n), cudaMemcpyHostToDevice, c->stream));
            off += es[k] * n;
        }
        if (n > 0 && c->ids[c->cur])
            OHPIC_CUDA_TRY(c, cudaMemcpyAsync(c->ids[c->cur] + c->seg[s], p + off, sizeof(uint32_t) * n,
                                              cudaMemcpyHostToDevice, c->stream));
        c->count[s] = n;
        if (!f64 && n > 0) {
            const int64_t blocks = std::min<int64_t>((n + 255) / 256, 152 * 16);
            k_check_restored<<<(unsigned)blocks, 256, 0, c->stream>>>(c->p32[c->cur], c->seg[s], n, c->cfg.nx,
                                                                      c->cfg.ny, c->cfg.nz, c->diag);
        }
        p += snap_species_bytes(f64, n);
    }
    OHPIC_CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    {
        const int rc = check_device(c);
        if (rc != OHPIC_OK) {
            // refuse the image and leave no particle that a kernel could misread
            for (int s = 0; s < c->cfg.nspecies; ++s) c->count[s] = 0;
            return fail(c, OHPIC_ERR_INVALID,
                        "snapshot_load: a particle lies outside the grid, has an offset outside [0, 1) or a "
                        "non-finite value (" + c->err + ")");
        }
    }
    c->steps = h.steps;
    c->steps_since_sort = h.steps_since_sort;
    c->sorted = false;        // the next step sorts, then deposits the restored particles
    c->rho_valid = false;
    c->field_valid = false;
    c->kin_valid = false;
    return check_device(c);
}

}  // extern "C"
