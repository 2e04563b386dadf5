// serve.cu -- continuous batching of many small periodic runs on one GPU.
//
// No reference counterpart: the reference advances one simulation per job
// (src/ohhelppic3d.f90:311-358).  Here one worker thread keeps every admitted
// run resident and advances all of them one step per tick:
//
//   fields     runs of one grid size share a FieldPool (fields.cu): slot k of the
//              pool is one run's rho/phi/spectrum/padded E/weight sums.  One batched
//              cuFFT plan pair and three pooled kernels solve every slot at once.
//   particles  one persistent launch of tiled_f32_multi (push_f32.cu) over all
//              runs: CTAs pull (run, species, tile) items from one queue ordered
//              by decreasing particles per item.
//   sort       every sort_every ticks, one histogram, one scan, one record scatter
//              and one transpose over every (run, species) segment (sort.cu); the
//              counters of all segments live in one key space laid out by pool slot.
//
// A tick's launches are captured into a CUDA graph (and a second graph for the
// sort) and replayed until the set of grid-size pools in use changes: the tables
// the kernels read (run and segment counts, run descriptors, item prefix, sort
// segments, pool slot masks) live in device memory and are refreshed by
// stream-ordered copies from pinned staging before the tick that needs them,
// and every grid is fixed, so admissions and retirements need no new capture.
//
// Admission: a run is admitted first-come first-served when its HBM footprint
// (particles twice for the sort, tile table, kept-result staging) and, for a new
// grid size, a new pool fit the budget.  It is drawn on the device with the
// injector of ohpic_init_particles, sorted and deposited (same multi-run
// kernels, admitted runs only) and joins the next tick.  A run that reaches its
// step count is retired right after its last tick in stream order (final rho,
// field and kinetic sums, kept arrays), its slot is released, and its memory is
// freed once the host has copied the result.
//
// Independence: the deposit is integer fixed point, every particle advances on
// its own, and a slot's transform is the same batched plan whatever the other
// slots hold, so a run's arrays do not depend on its neighbours or its slot.
// Only FP64 atomic sums (charge, energies) may differ in the last bits.
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "ohpic_internal.cuh"
#include "../../include/ohpic_serve.h"

using namespace ohpic;

namespace {

constexpr int kDepth = 2;          // ticks in flight
constexpr int kStageSlots = 4;     // pinned staging buffers for table uploads

int64_t align256(int64_t v) { return (v + 255) & ~(int64_t)255; }

// Tile edge for a grid edge n: the largest power of two <= want (8 when want is 0)
// that divides n, so one setting serves every grid size.
int pick_tile(int n, int want)
{
    int t = 1;
    while (2 * t <= (want > 0 ? want : 8)) t *= 2;
    for (; t > 1; t >>= 1)
        if (n % t == 0) return t;
    return 1;
}

// ---- device helpers for retirement ----

// Kinetic sums (|v|^2, vx, vy, vz) of one species into out4 (FP64 atomics).
__global__ void k_run_kinetic(PartF32 p, int64_t seg, int64_t n, double *out4)
{
    double ke = 0, mx = 0, my = 0, mz = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double vx = p.vx[seg + i], vy = p.vy[seg + i], vz = p.vz[seg + i];
        ke += vx * vx + vy * vy + vz * vz;
        mx += vx; my += vy; mz += vz;
    }
    for (int o = 16; o > 0; o >>= 1) {
        ke += __shfl_xor_sync(0xffffffffu, ke, o);
        mx += __shfl_xor_sync(0xffffffffu, mx, o);
        my += __shfl_xor_sync(0xffffffffu, my, o);
        mz += __shfl_xor_sync(0xffffffffu, mz, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(out4 + 0, ke);
        atomicAdd(out4 + 1, mx);
        atomicAdd(out4 + 2, my);
        atomicAdd(out4 + 3, mz);
    }
}

// Particles of one species in injection order (ids are the injector's indices):
// out holds 6 blocks of n doubles (x, y, z, vx, vy, vz).
__global__ void k_run_by_id(PartF32 p, const uint32_t *ids, int64_t seg, int64_t n, double *out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = seg + i;
        const int64_t k = ids[o];
        if (k >= n) continue;
        const int32_t c = p.cell[o];
        out[k] = (double)cell_x(c) + (double)p.ox[o];
        out[n + k] = (double)cell_y(c) + (double)p.oy[o];
        out[2 * n + k] = (double)cell_z(c) + (double)p.oz[o];
        out[3 * n + k] = p.vx[o];
        out[4 * n + k] = p.vy[o];
        out[5 * n + k] = p.vz[o];
    }
}

int grid_for(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > 152 * 8) b = 152 * 8;
    return b < 1 ? 1 : (int)b;
}

// ---- host state ----

struct Pool {
    FieldPool f{};
    int n[3] = {0, 0, 0};
    std::vector<int64_t> owner;   // run id per slot, -1 when free
    std::vector<double> q;        // host mirror of f.q
    std::vector<int> on;          // host mirror of f.on
    int used = 0;
    int64_t key_base = 0;         // first sort counter of slot 0
    int64_t bytes = 0;
    bool plans = false;
};

struct Run {
    int64_t id = 0;
    ohpic_run_request req{};
    int nsp = 0;
    int64_t count[OHPIC_MAX_SPECIES] = {0};
    int64_t seg[OHPIC_MAX_SPECIES] = {0};
    int64_t total = 0;            // particles
    int64_t slots = 0;            // particle array length (segments 64-aligned)
    int64_t bytes = 0;            // device bytes held from admission to release
    int64_t out_doubles = 0;      // kept fields + particles
    void *mem = nullptr;
    PartF32 p{};                  // the particles, sorted in place
    uint32_t *ids = nullptr;      // with keep_particles
    int4 *rec = nullptr;          // sort record area, 32 bytes per slot
    int64_t *tile_begin = nullptr;
    DevDiag *diag = nullptr;
    double *out = nullptr;
    Pool *pool = nullptr;
    int slot = -1;
    Geom g{};
    SpeciesConst sc[OHPIC_MAX_SPECIES]{};
    int64_t steps = 0;
    int64_t items = 0;
    double t_submit = 0, t_admit = 0, t_finish = 0;
    int status = OHPIC_OK;
    bool done = false;
    cudaEvent_t ev = nullptr;     // recorded after the retirement work
    std::vector<double> fields, parts;
    ohpic_diag diag_out{};
};

// Byte layout of a run's single allocation.
struct RunLayout {
    int64_t p, ids, rec, tile_begin, diag, out, total;
};

RunLayout run_layout(int64_t slots, int nsp, int64_t ntile, bool ids, int64_t out_doubles)
{
    RunLayout L{};
    int64_t off = 0;
    const int64_t part = align256(slots * 4);
    L.p = off; off += 7 * part;
    L.ids = off; off += ids ? part : 0;
    L.rec = off; off += align256(slots * 32);
    L.tile_begin = off; off += align256((int64_t)nsp * (ntile + 1) * 8);
    L.diag = off; off += align256((int64_t)sizeof(DevDiag));
    L.out = off; off += align256(out_doubles * 8);
    L.total = off;
    return L;
}

PartF32 part_view(unsigned char *base, int64_t slots)
{
    const int64_t part = align256(slots * 4);
    PartF32 p;
    p.cell = (int32_t *)base;
    p.ox = (float *)(base + part);
    p.oy = (float *)(base + 2 * part);
    p.oz = (float *)(base + 3 * part);
    p.vx = (float *)(base + 4 * part);
    p.vy = (float *)(base + 5 * part);
    p.vz = (float *)(base + 6 * part);
    return p;
}

// Pool field bytes for one grid size.
int64_t pool_bytes(const Geom &g, int slots, int nsp)
{
    const int64_t npad = (int64_t)g.gx * g.gy * g.gz;
    int64_t b = 0;
    b += align256(slots * g.ncell * 4) * 2;                 // rho, phi
    b += align256(slots * g.nspec * 8);                     // spectrum
    b += align256(slots * npad * 16);                       // padded E
    b += align256((int64_t)slots * nsp * g.ncell * 8);      // weight sums
    b += align256(g.nspec * 8);                             // green
    b += align256((int64_t)slots * nsp * 8) + align256(slots * 4);
    return b;
}

}  // namespace

struct ohpic_server {
    ohpic_serve_config cfg{};
    int dev = 0;
    int sms = 152;
    cudaStream_t st = nullptr;
    cudaMemPool_t mempool = nullptr;
    std::chrono::steady_clock::time_point t0;

    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;                                 // under mu
    std::deque<Run *> incoming;                        // under mu
    std::map<int64_t, std::unique_ptr<Run>> runs;      // under mu
    std::deque<int64_t> completed;                     // under mu: not yet polled
    int64_t next_id = 1;                               // under mu
    int64_t outstanding = 0;                           // under mu: submitted, not final
    ohpic_serve_stats stats{};                         // under mu
    std::string err;                                   // under mu
    bool dead = false;                                 // under mu: the worker stopped on a CUDA error

    // worker thread only
    std::deque<Run *> pending;
    std::vector<Run *> active, retiring;
    std::vector<std::unique_ptr<Pool>> pools;
    int64_t bytes_in_use = 0;
    int64_t nkeys = 0, nkeys_cap = 0;
    uint32_t *d_count = nullptr, *d_start = nullptr, *d_cur32 = nullptr, *d_scan_tmp = nullptr;
    RunDesc *d_runs = nullptr;
    int64_t *d_item_end = nullptr;
    SortSeg *d_segs = nullptr;
    int32_t *d_chunk_end = nullptr;
    unsigned long long *d_cursor = nullptr;
    int *d_nums = nullptr;                             // [0] runs, [1] sort segments of the tables
    unsigned char *h_stage[kStageSlots] = {};
    cudaEvent_t stage_ev[kStageSlots] = {};
    bool stage_used[kStageSlots] = {};
    int stage_next = 0;
    size_t stage_bytes = 0;
    cudaEvent_t tick_ev[kDepth] = {};
    int64_t ticks = 0;
    int ticks_since_sort = 0;
    // shapes of the uploaded tables
    int tab_nruns = 0, tab_nseg = 0;
    int64_t tab_items = 0, tab_chunks = 0, tab_max_ntile = 0, tab_particles = 0;
    size_t push_smem = 0;
    int push_grid = 0;
    bool shapes_dirty = true;
    // The graphs depend only on the pools in use and the key space: run and
    // segment counts are read from device memory and the grids are fixed.
    std::vector<int> graph_pools;
    int64_t graph_nkeys = -1;
    cudaGraphExec_t g_tick = nullptr, g_sort = nullptr;
    int64_t launches_tick = 0, launches_sort = 0;

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    void set_err(const std::string &m)
    {
        std::lock_guard<std::mutex> lk(mu);
        err = m;
    }
};

namespace {

using Server = ohpic_server;

// Geometry of a run's grid with the server's tile and halo (FP32 form).
// Largest tile edges: y and z, then x.
void tile_edges(const ohpic_serve_config &cfg, int &t, int &tx)
{
    t = cfg.tile > 0 ? cfg.tile : 8;
    tx = cfg.tile_x > 0 ? cfg.tile_x : std::min(64, 2 * t);
}

bool serve_geom(const ohpic_serve_config &cfg, int nx, int ny, int nz, Geom &g)
{
    ohpic_config k;
    ohpic_config_default(&k);
    k.nx = nx; k.ny = ny; k.nz = nz;
    k.precision = OHPIC_FP32;
    int t, tx;
    tile_edges(cfg, t, tx);
    const int tile[3] = {pick_tile(nx, tx), pick_tile(ny, t), pick_tile(nz, t)};
    if (tile[0] < 1 || tile[1] < 1 || tile[2] < 1) return false;
    return make_geom(k, tile, cfg.halo, g);
}

// Allocation on the server's stream-ordered pool.
template <typename T>
bool salloc(Server *s, T **p, int64_t bytes)
{
    *p = nullptr;
    if (bytes <= 0) bytes = 256;
    if (cudaMallocFromPoolAsync((void **)p, (size_t)bytes, s->mempool, s->st) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return false;
    }
    return true;
}

void sfree(Server *s, void *p)
{
    if (p) cudaFreeAsync(p, s->st);
}

// Grows the sort key arrays to the key space of every pool.
bool ensure_keys(Server *s)
{
    if (s->nkeys <= s->nkeys_cap) return true;
    sfree(s, s->d_count);
    sfree(s, s->d_start);
    sfree(s, s->d_cur32);
    sfree(s, s->d_scan_tmp);
    s->d_count = s->d_start = s->d_cur32 = s->d_scan_tmp = nullptr;
    const int64_t n = s->nkeys;
    if (!salloc(s, &s->d_count, n * 4) || !salloc(s, &s->d_start, n * 4) || !salloc(s, &s->d_cur32, n * 4) ||
        !salloc(s, &s->d_scan_tmp, scan_tmp_elems(n) * 4)) {
        s->nkeys_cap = 0;
        return false;
    }
    s->nkeys_cap = n;
    s->shapes_dirty = true;
    return true;
}

Pool *create_pool(Server *s, const Geom &g, std::string &why)
{
    std::unique_ptr<Pool> P(new Pool());
    const int slots = s->cfg.slots_per_pool, nsp = s->cfg.max_species;
    P->n[0] = g.nx; P->n[1] = g.ny; P->n[2] = g.nz;
    FieldPool &f = P->f;
    f.g = g;
    f.slots = slots;
    f.nsp = nsp;
    const int64_t npad = (int64_t)g.gx * g.gy * g.gz;
    bool ok = salloc(s, &f.rho, slots * g.ncell * 4) && salloc(s, &f.phi, slots * g.ncell * 4) &&
              salloc(s, &f.spec, slots * g.nspec * 8) && salloc(s, &f.epad, slots * npad * 16) &&
              salloc(s, &f.wsum, (int64_t)slots * nsp * g.ncell * 8) && salloc(s, &f.green, g.nspec * 8) &&
              salloc(s, &f.q, (int64_t)slots * nsp * 8) && salloc(s, &f.on, (int64_t)slots * 4);
    if (ok) {
        cudaMemsetAsync(f.rho, 0, slots * g.ncell * 4, s->st);
        cudaMemsetAsync(f.phi, 0, slots * g.ncell * 4, s->st);
        cudaMemsetAsync(f.epad, 0, slots * npad * 16, s->st);
        cudaMemsetAsync(f.wsum, 0, (size_t)slots * nsp * g.ncell * 8, s->st);
        cudaMemsetAsync(f.q, 0, (size_t)slots * nsp * 8, s->st);
        cudaMemsetAsync(f.on, 0, (size_t)slots * 4, s->st);
        pool_green(s->st, g, f.green);
        int dims[3] = {g.nz, g.ny, g.nx};
        ok = cufftPlanMany(&f.r2c, 3, dims, nullptr, 1, (int)g.ncell, nullptr, 1, (int)g.nspec, CUFFT_R2C, slots) ==
             CUFFT_SUCCESS;
        if (ok) {
            ok = cufftPlanMany(&f.c2r, 3, dims, nullptr, 1, (int)g.nspec, nullptr, 1, (int)g.ncell, CUFFT_C2R,
                               slots) == CUFFT_SUCCESS;
            if (!ok) cufftDestroy(f.r2c);
        }
        if (ok) {
            P->plans = true;
            cufftSetStream(f.r2c, s->st);
            cufftSetStream(f.c2r, s->st);
        } else {
            why = "cufftPlanMany failed";
        }
    } else {
        why = "pool allocation failed";
    }
    if (!ok) {
        for (void *p : {(void *)f.rho, (void *)f.phi, (void *)f.spec, (void *)f.epad, (void *)f.wsum, (void *)f.green,
                        (void *)f.q, (void *)f.on})
            sfree(s, p);
        return nullptr;
    }
    size_t w1 = 0, w2 = 0;
    cufftGetSize(f.r2c, &w1);
    cufftGetSize(f.c2r, &w2);
    P->bytes = pool_bytes(g, slots, nsp) + (int64_t)(w1 + w2);
    P->owner.assign(slots, -1);
    P->q.assign((size_t)slots * nsp, 0.0);
    P->on.assign(slots, 0);
    P->key_base = s->nkeys;
    s->nkeys += (int64_t)slots * nsp * g.ncell;
    s->bytes_in_use += P->bytes;
    s->pools.push_back(std::move(P));
    s->shapes_dirty = true;
    return s->pools.back().get();
}

void destroy_pool(Server *s, Pool *P)
{
    FieldPool &f = P->f;
    if (P->plans) {
        cufftDestroy(f.r2c);
        cufftDestroy(f.c2r);
        P->plans = false;
    }
    for (void *p : {(void *)f.rho, (void *)f.phi, (void *)f.spec, (void *)f.epad, (void *)f.wsum, (void *)f.green,
                    (void *)f.q, (void *)f.on})
        sfree(s, p);
}

// Run descriptor for the multi-run push.
RunDesc make_desc(const Server *s, const Run *r)
{
    RunDesc d;
    memset(&d, 0, sizeof(d));
    TileArgs &a = d.a;
    const Pool &P = *r->pool;
    a.g = r->g;
    a.nspecies = r->nsp;
    a.weights = s->cfg.weights;
    a.split = 1;
    a.deposit = s->cfg.deposit;
    a.use_tma = 0;
    a.with_energy = 0;
    a.sorted = 1;
    a.ppl = s->cfg.lane_particles;
    for (int k = 0; k < r->nsp; ++k) {
        a.seg[k] = r->seg[k];
        a.count[k] = r->count[k];
        a.sc[k] = r->sc[k];
    }
    const int64_t npad = (int64_t)r->g.gx * r->g.gy * r->g.gz;
    a.tile_begin = r->tile_begin;
    a.epad = P.f.epad + (int64_t)r->slot * npad;
    a.rho = nullptr;
    a.wsum = P.f.wsum + (int64_t)r->slot * P.f.nsp * r->g.ncell;
    a.interp_out = nullptr;
    a.diag = r->diag;
    a.chunk = 4096;
    d.p = r->p;
    return d;
}

// A pinned staging buffer whose previous copy has completed.
unsigned char *stage_take(Server *s, int &slot)
{
    slot = s->stage_next;
    s->stage_next = (s->stage_next + 1) % kStageSlots;
    if (s->stage_used[slot]) cudaEventSynchronize(s->stage_ev[slot]);
    return s->h_stage[slot];
}

void stage_done(Server *s, int slot)
{
    cudaEventRecord(s->stage_ev[slot], s->st);
    s->stage_used[slot] = true;
}

// Uploads the tables of `runs` (in queue order: decreasing particles per item)
// and the slot masks of every pool.  Sets the launch shapes.
bool upload_tables(Server *s, std::vector<Run *> &runs)
{
    std::stable_sort(runs.begin(), runs.end(), [](const Run *x, const Run *y) {
        return (double)x->total / (double)std::max<int64_t>(x->items, 1) >
               (double)y->total / (double)std::max<int64_t>(y->items, 1);
    });
    const int n = (int)runs.size();
    int nseg = 0;
    for (const Run *r : runs) nseg += r->nsp;
    if (n > kMaxServeRuns || nseg > kMaxSortSegs) return false;
    size_t off = 0;
    const size_t o_runs = off; off += align256((int64_t)sizeof(RunDesc) * n);
    const size_t o_end = off; off += align256(8 * (int64_t)n);
    const size_t o_segs = off; off += align256((int64_t)sizeof(SortSeg) * nseg);
    const size_t o_chunk = off; off += align256(4 * (int64_t)nseg);
    const size_t o_nums = off; off += 256;
    const size_t o_pools = off;
    for (const auto &P : s->pools) off += align256(P->q.size() * 8) + align256(P->on.size() * 4);
    if (off > s->stage_bytes) return false;
    int slot;
    unsigned char *h = stage_take(s, slot);
    RunDesc *hr = (RunDesc *)(h + o_runs);
    int64_t *he = (int64_t *)(h + o_end);
    SortSeg *hs = (SortSeg *)(h + o_segs);
    int32_t *hc = (int32_t *)(h + o_chunk);
    int64_t items = 0, chunks = 0, max_nt = 0, parts = 0;
    int si = 0;
    for (int i = 0; i < n; ++i) {
        Run *r = runs[i];
        hr[i] = make_desc(s, r);
        items += r->items;
        he[i] = items;
        parts += r->total;
        max_nt = std::max<int64_t>(max_nt, r->g.ntile);
        const Pool &P = *r->pool;
        for (int k = 0; k < r->nsp; ++k, ++si) {
            SortSeg &sg = hs[si];
            memset(&sg, 0, sizeof(sg));
            sg.g = r->g;
            sg.p = r->p;
            sg.ids = r->ids;
            sg.rec = r->rec;
            sg.off = r->seg[k];
            sg.count = r->count[k];
            sg.key_base = P.key_base + ((int64_t)r->slot * P.f.nsp + k) * r->g.ncell;
            sg.tile_begin = r->tile_begin + (int64_t)k * (r->g.ntile + 1);
            sg.diag = r->diag;
            sg.h = s->cfg.sort_lead > 0 ? (float)(s->cfg.sort_lead * r->sc[k].dt) : 0.f;
            chunks += (r->count[k] + kSortChunk - 1) / kSortChunk;
            hc[si] = (int32_t)chunks;
        }
    }
    size_t po = o_pools;
    for (const auto &P : s->pools) {
        memcpy(h + po, P->q.data(), P->q.size() * 8);
        cudaMemcpyAsync(P->f.q, h + po, P->q.size() * 8, cudaMemcpyHostToDevice, s->st);
        po += align256(P->q.size() * 8);
        memcpy(h + po, P->on.data(), P->on.size() * 4);
        cudaMemcpyAsync(P->f.on, h + po, P->on.size() * 4, cudaMemcpyHostToDevice, s->st);
        po += align256(P->on.size() * 4);
    }
    if (n > 0) {
        cudaMemcpyAsync(s->d_runs, hr, sizeof(RunDesc) * n, cudaMemcpyHostToDevice, s->st);
        cudaMemcpyAsync(s->d_item_end, he, 8 * (size_t)n, cudaMemcpyHostToDevice, s->st);
    }
    if (nseg > 0) {
        cudaMemcpyAsync(s->d_segs, hs, sizeof(SortSeg) * nseg, cudaMemcpyHostToDevice, s->st);
        cudaMemcpyAsync(s->d_chunk_end, hc, 4 * (size_t)nseg, cudaMemcpyHostToDevice, s->st);
    }
    int *hn = (int *)(h + o_nums);
    hn[0] = n;
    hn[1] = nseg;
    cudaMemcpyAsync(s->d_nums, hn, 2 * sizeof(int), cudaMemcpyHostToDevice, s->st);
    stage_done(s, slot);
    s->tab_nruns = n;
    s->tab_nseg = nseg;
    s->tab_items = items;
    s->tab_chunks = chunks;
    s->tab_max_ntile = max_nt;
    s->tab_particles = parts;
    return true;
}

// Launch shapes that do not depend on the set of runs: the persistent push and
// the sort passes loop over whatever the tables hold.
void fixed_shapes(Server *s)
{
    Geom g;
    int t, tx;
    tile_edges(s->cfg, t, tx);
    const int n = 2 * std::max(t, tx);   // the largest staged box any grid gets
    serve_geom(s->cfg, n, n, n, g);
    s->push_smem = (size_t)((((int64_t)g.sx * g.sy * g.sz * (16 + 8) + 15) & ~(int64_t)15) + 128 +
                            (s->cfg.lane_particles == 4 ? kQuadStageBytes : 0));
    s->push_grid = s->sms * 2;
    int64_t nt = 0;
    for (const auto &P : s->pools) nt = std::max<int64_t>(nt, P->f.g.ntile);
    s->tab_max_ntile = nt;
}

MultiPush multi_push(const Server *s)
{
    MultiPush m;
    m.runs = s->d_runs;
    m.item_end = s->d_item_end;
    m.nruns = s->d_nums;
    m.cursor = s->d_cursor;
    return m;
}

MultiSort multi_sort(const Server *s)
{
    MultiSort m;
    m.segs = s->d_segs;
    m.chunk_end = s->d_chunk_end;
    m.nseg = s->d_nums + 1;
    m.count = s->d_count;
    m.start = s->d_start;
    m.cursor = s->d_cur32;
    return m;
}

// The cell sort of the segments in the tables; returns launches (memsets count
// as launches).  Grids are fixed; the kernels loop over the uploaded chunks.
int64_t enqueue_sort(Server *s)
{
    fixed_shapes(s);
    const MultiSort m = multi_sort(s);
    const int64_t grid = (int64_t)s->sms * 8;
    int64_t l = 2;
    cudaMemsetAsync(s->d_count, 0, (size_t)s->nkeys * 4, s->st);
    l += launch_sort_hist_multi(s->st, m, grid);
    cudaMemsetAsync(s->d_cur32, 0, (size_t)s->nkeys * 4, s->st);
    l += launch_sort_finish_multi(s->st, m, grid, s->tab_max_ntile, kMaxSortSegs, s->nkeys, s->d_scan_tmp);
    return l;
}

// The field solve of every pool in use, then the push (or the deposit) of the
// runs in the tables; returns launches, -1 on a cuFFT or launch error.
int64_t enqueue_step(Server *s, int mode)
{
    fixed_shapes(s);
    int64_t l = 0;
    if (mode == MODE_PUSH) {
        for (const auto &P : s->pools) {
            if (P->used == 0) continue;
            const int k = pool_solve(s->st, P->f);
            if (k < 0) return -1;
            l += k;
        }
    }
    cudaMemsetAsync(s->d_cursor, 0, sizeof(unsigned long long), s->st);
    if (launch_multi_f32(s->st, mode, s->cfg.deposit, s->cfg.lane_particles, s->cfg.weights, multi_push(s),
                         s->push_grid,
                         s->push_smem) != cudaSuccess)
        return -1;
    return l + 2;
}

}  // namespace

namespace {

// Marks a run final (under the lock) and wakes waiters.
void publish(Server *s, Run *r, int status)
{
    std::lock_guard<std::mutex> lk(s->mu);
    r->status = status;
    r->done = true;
    r->t_finish = s->now();
    s->completed.push_back(r->id);
    s->stats.completed += 1;
    if (status != OHPIC_OK) s->stats.failed += 1;
    s->outstanding -= 1;
    s->cv_done.notify_all();
}

void release_slot(Server *s, Run *r)
{
    Pool &P = *r->pool;
    P.owner[r->slot] = -1;
    P.on[r->slot] = 0;
    for (int k = 0; k < P.f.nsp; ++k) P.q[(size_t)r->slot * P.f.nsp + k] = 0.0;
    P.used -= 1;
    (void)s;
}

// Enqueues the final-state work of a run after its last tick and releases its
// field slot (later users of the slot are ordered after this work).
void retire_enqueue(Server *s, Run *r)
{
    const Pool &P = *r->pool;
    const Geom &g = r->g;
    pool_slot_rho(s->st, P.f, r->slot);
    pool_slot_sums(s->st, P.f, r->slot, r->diag);
    cudaMemsetAsync(r->diag->kin, 0, sizeof(r->diag->kin), s->st);
    for (int k = 0; k < r->nsp; ++k)
        if (r->count[k] > 0)
            k_run_kinetic<<<grid_for(r->count[k]), 256, 0, s->st>>>(r->p, r->seg[k], r->count[k],
                                                                    &r->diag->kin[k][0]);
    int64_t off = 0;
    if (r->req.keep_fields) {
        pool_slot_fields(s->st, P.f, r->slot, r->out);
        off += 5 * g.ncell;
    }
    if (r->req.keep_particles) {
        for (int k = 0; k < r->nsp; ++k) {
            if (r->count[k] > 0)
                k_run_by_id<<<grid_for(r->count[k]), 256, 0, s->st>>>(r->p, r->ids, r->seg[k],
                                                                      r->count[k], r->out + off);
            off += 6 * r->count[k];
        }
    }
    cudaEventCreateWithFlags(&r->ev, cudaEventDisableTiming);
    cudaEventRecord(r->ev, s->st);
    release_slot(s, r);
    s->retiring.push_back(r);
    s->shapes_dirty = true;
}

// Copies the results of retired runs whose work has completed and frees their
// memory; with block, waits for the oldest one.
void finish_retired(Server *s, bool block)
{
    for (size_t i = 0; i < s->retiring.size();) {
        Run *r = s->retiring[i];
        cudaError_t q = (block && i == 0) ? cudaEventSynchronize(r->ev) : cudaEventQuery(r->ev);
        if (q == cudaErrorNotReady) {
            ++i;
            continue;
        }
        int status = q == cudaSuccess ? OHPIC_OK : OHPIC_ERR_CUDA;
        DevDiag h;
        memset(&h, 0, sizeof(h));
        if (status == OHPIC_OK && cudaMemcpy(&h, r->diag, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess)
            status = OHPIC_ERR_CUDA;
        if (status == OHPIC_OK && h.err_code != 0) status = h.err_code;
        ohpic_diag &d = r->diag_out;
        memset(&d, 0, sizeof(d));
        for (int k = 0; k < r->nsp; ++k) {
            d.count[k] = r->count[k];
            const double m = r->req.q[k] / r->req.qm[k];
            d.kinetic_energy += 0.5 * m * h.kin[k][0];
            for (int c = 0; c < 3; ++c) d.momentum[c] += m * h.kin[k][1 + c];
        }
        for (int c = 0; c < 3; ++c) d.crossings[c] = (int64_t)h.crossings[c];
        d.outside_tile = (int64_t)h.outside;
        d.step = r->steps;
        d.total_charge = h.charge;
        d.field_energy = h.field_energy;
        if (status == OHPIC_OK && r->out_doubles > 0) {
            const int64_t nf = r->req.keep_fields ? 5 * r->g.ncell : 0;
            if (nf > 0) {
                r->fields.resize((size_t)nf);
                if (cudaMemcpy(r->fields.data(), r->out, (size_t)nf * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
                    status = OHPIC_ERR_CUDA;
            }
            const int64_t np = r->out_doubles - nf;
            if (np > 0 && status == OHPIC_OK) {
                r->parts.resize((size_t)np);
                if (cudaMemcpy(r->parts.data(), r->out + nf, (size_t)np * 8, cudaMemcpyDeviceToHost) != cudaSuccess)
                    status = OHPIC_ERR_CUDA;
            }
        }
        cudaEventDestroy(r->ev);
        r->ev = nullptr;
        sfree(s, r->mem);
        r->mem = nullptr;
        s->bytes_in_use -= r->bytes;
        s->retiring.erase(s->retiring.begin() + (long)i);
        publish(s, r, status);
        block = false;
    }
}

// Admits pending runs first-come first-served while they fit; draws, sorts and
// deposits the admitted runs together.
bool admit(Server *s)
{
    std::vector<Run *> fresh;
    int nseg = 0;
    int64_t parts = 0;   // the sort scans 32-bit counters over every active particle
    for (const Run *r : s->active) {
        nseg += r->nsp;
        parts += r->total;
    }
    while (!s->pending.empty() && (int)(s->active.size() + fresh.size()) < s->cfg.max_active) {
        Run *r = s->pending.front();
        if (nseg + r->nsp > kMaxSortSegs || parts + r->total >= (int64_t)UINT32_MAX) break;
        Pool *P = nullptr;
        for (const auto &q : s->pools)
            if (q->n[0] == r->req.nx && q->n[1] == r->req.ny && q->n[2] == r->req.nz && q->used < q->f.slots) {
                P = q.get();
                break;
            }
        const int64_t extra = P ? 0 : pool_bytes(r->g, s->cfg.slots_per_pool, s->cfg.max_species);
        if (s->bytes_in_use + r->bytes + extra > s->cfg.hbm_budget) {
            const bool alone = s->active.empty() && fresh.empty() && s->retiring.empty();
            if (!alone) break;   // wait for memory to free up
            s->pending.pop_front();
            publish(s, r, OHPIC_ERR_CAPACITY);
            continue;
        }
        std::string why;
        if (!P) P = create_pool(s, r->g, why);
        if (!P || !ensure_keys(s)) {
            s->pending.pop_front();
            s->set_err(P ? "sort key allocation failed" : why);
            publish(s, r, OHPIC_ERR_OOM);
            continue;
        }
        if (!salloc(s, (unsigned char **)&r->mem, r->bytes)) {
            if (!s->active.empty() || !fresh.empty() || !s->retiring.empty()) break;
            s->pending.pop_front();
            publish(s, r, OHPIC_ERR_OOM);
            continue;
        }
        s->pending.pop_front();
        unsigned char *base = (unsigned char *)r->mem;
        const bool ids = r->req.keep_particles != 0;
        const RunLayout L = run_layout(r->slots, r->nsp, r->g.ntile, ids, r->out_doubles);
        r->p = part_view(base + L.p, r->slots);
        r->ids = ids ? (uint32_t *)(base + L.ids) : nullptr;
        r->rec = (int4 *)(base + L.rec);
        r->tile_begin = (int64_t *)(base + L.tile_begin);
        r->diag = (DevDiag *)(base + L.diag);
        r->out = (double *)(base + L.out);
        int slot = 0;
        while (P->owner[slot] >= 0) ++slot;
        r->pool = P;
        r->slot = slot;
        P->owner[slot] = r->id;
        P->on[slot] = 1;
        for (int k = 0; k < r->nsp; ++k) P->q[(size_t)slot * P->f.nsp + k] = r->req.q[k];
        P->used += 1;
        s->bytes_in_use += r->bytes;
        cudaMemsetAsync(r->diag, 0, sizeof(DevDiag), s->st);
        cudaMemsetAsync(P->f.wsum + (int64_t)slot * P->f.nsp * r->g.ncell, 0,
                        (size_t)P->f.nsp * r->g.ncell * 8, s->st);
        DrawSpec d;
        d.stream = s->st;
        d.precision = OHPIC_FP32;
        d.n[0] = r->req.nx; d.n[1] = r->req.ny; d.n[2] = r->req.nz;
        d.initstate = r->req.seed_state;
        d.initseq = r->req.seed_seq;
        d.advance = 0;
        d.nspecies = r->nsp;
        d.spi = r->req.species;
        d.seg = r->seg;
        d.cap = nullptr;
        d.p32 = r->p;
        d.ids = r->ids;
        int64_t cnt[OHPIC_MAX_SPECIES] = {0};
        draw_particles(d, cnt, nullptr);
        r->steps = 0;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            r->t_admit = s->now();
            s->stats.admitted += 1;
        }
        nseg += r->nsp;
        parts += r->total;
        fresh.push_back(r);
    }
    if (fresh.empty()) return true;
    // Sort, then deposit, the admitted runs only (the push of the next tick needs
    // their weight sums); the tick tables are rebuilt afterwards.
    if (!upload_tables(s, fresh)) return false;
    const int64_t l = enqueue_sort(s);
    const int64_t l2 = enqueue_step(s, MODE_DEPOSIT);
    if (l2 < 0) return false;
    for (Run *r : fresh) s->active.push_back(r);
    s->shapes_dirty = true;
    std::lock_guard<std::mutex> lk(s->mu);
    s->stats.launches += l + l2;
    return true;
}

bool capture(Server *s, bool sort, cudaGraphExec_t *out, int64_t *launches)
{
    if (*out) {
        cudaGraphExecDestroy(*out);
        *out = nullptr;
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(s->st, cudaStreamCaptureModeRelaxed) != cudaSuccess) return false;
    const int64_t l = sort ? enqueue_sort(s) : enqueue_step(s, MODE_PUSH);
    const cudaError_t e = cudaStreamEndCapture(s->st, &g);
    if (e != cudaSuccess || l < 0 || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return false;
    }
    const cudaError_t e2 = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e2 != cudaSuccess) {
        *out = nullptr;
        cudaGetLastError();
        return false;
    }
    *launches = l;
    std::lock_guard<std::mutex> lk(s->mu);
    s->stats.graph_captures += 1;
    return true;
}

// One step of every active run: (sort,) field solve of every pool, push.
bool tick(Server *s)
{
    const int idx = (int)(s->ticks % kDepth);
    if (s->ticks >= kDepth) cudaEventSynchronize(s->tick_ev[idx]);
    const bool sort_now = s->cfg.sort_every > 0 && s->ticks_since_sort >= s->cfg.sort_every;
    // the sort works in place, so the tables change only with the set of runs
    if (s->shapes_dirty) {
        if (!upload_tables(s, s->active)) return false;
    }
    int64_t launched = 0;
    bool via_graph = false;
    if (s->cfg.use_graphs) {
        std::vector<int> in_use;
        for (size_t i = 0; i < s->pools.size(); ++i)
            if (s->pools[i]->used > 0) in_use.push_back((int)i);
        bool ok = true;
        if (in_use != s->graph_pools || s->graph_nkeys != s->nkeys || !s->g_tick || !s->g_sort) {
            ok = capture(s, false, &s->g_tick, &s->launches_tick) && capture(s, true, &s->g_sort, &s->launches_sort);
            if (ok) {
                s->graph_pools = in_use;
                s->graph_nkeys = s->nkeys;
            } else {
                s->graph_pools.clear();
                s->graph_nkeys = -1;
            }
        }
        if (ok && s->g_tick && s->g_sort) {
            if (sort_now) {
                if (cudaGraphLaunch(s->g_sort, s->st) != cudaSuccess) return false;
                launched += s->launches_sort;
            }
            if (cudaGraphLaunch(s->g_tick, s->st) != cudaSuccess) return false;
            launched += s->launches_tick;
            via_graph = true;
        }
    }
    if (!via_graph) {
        if (sort_now) launched += enqueue_sort(s);
        const int64_t l = enqueue_step(s, MODE_PUSH);
        if (l < 0) return false;
        launched += l;
    }
    s->shapes_dirty = false;
    if (sort_now) s->ticks_since_sort = 0;
    s->ticks_since_sort += 1;
    cudaEventRecord(s->tick_ev[idx], s->st);
    s->ticks += 1;
    int64_t psteps = 0;
    for (const Run *r : s->active) psteps += r->total;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stats.ticks += 1;
        s->stats.sort_ticks += sort_now ? 1 : 0;
        s->stats.particle_steps += psteps;
        s->stats.launches += launched;
        s->stats.graph_launches += via_graph ? (sort_now ? 2 : 1) : 0;
    }
    // Runs that reached their step count leave after this tick.
    std::vector<Run *> keep;
    keep.reserve(s->active.size());
    for (Run *r : s->active) {
        r->steps += 1;
        if (r->steps >= r->req.nsteps) retire_enqueue(s, r);
        else keep.push_back(r);
    }
    s->active.swap(keep);
    return cudaGetLastError() == cudaSuccess;
}

void fail_everything(Server *s, const std::string &why)
{
    cudaStreamSynchronize(s->st);
    cudaGetLastError();
    s->set_err(why);
    for (Run *r : s->retiring) {
        if (r->ev) cudaEventDestroy(r->ev);
        r->ev = nullptr;
        publish(s, r, OHPIC_ERR_CUDA);
    }
    s->retiring.clear();
    for (Run *r : s->active) publish(s, r, OHPIC_ERR_CUDA);
    s->active.clear();
    for (Run *r : s->pending) publish(s, r, OHPIC_ERR_CUDA);
    s->pending.clear();
    std::lock_guard<std::mutex> lk(s->mu);
    for (Run *r : s->incoming) {
        r->status = OHPIC_ERR_CUDA;
        r->done = true;
        s->completed.push_back(r->id);
        s->outstanding -= 1;
    }
    s->incoming.clear();
    s->dead = true;
    s->cv_done.notify_all();
}

void worker_main(Server *s)
{
    cudaSetDevice(s->dev);
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->active.empty() && s->retiring.empty() && s->pending.empty())
                s->cv_work.wait(lk, [&] { return s->stop || !s->incoming.empty(); });
            if (s->stop) break;
            while (!s->incoming.empty()) {
                s->pending.push_back(s->incoming.front());
                s->incoming.pop_front();
            }
            s->stats.pending = (int64_t)s->pending.size();
        }
        finish_retired(s, false);
        if (!admit(s)) {
            fail_everything(s, "admission failed: " + std::string(cudaGetErrorString(cudaGetLastError())));
            break;
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stats.active = (int64_t)s->active.size();
            s->stats.pending = (int64_t)s->pending.size();
            s->stats.bytes_in_use = s->bytes_in_use;
            s->stats.bytes_peak = std::max(s->stats.bytes_peak, s->bytes_in_use);
            s->stats.pools = (int32_t)s->pools.size();
        }
        if (s->active.empty()) {
            if (!s->retiring.empty()) finish_retired(s, true);
            continue;
        }
        if (!tick(s)) {
            fail_everything(s, "tick failed: " + std::string(cudaGetErrorString(cudaGetLastError())));
            break;
        }
    }
    cudaStreamSynchronize(s->st);
    finish_retired(s, false);
}

bool request_ok(const ohpic_serve_config &cfg, const ohpic_run_request &q)
{
    if (q.nx < 2 || q.ny < 2 || q.nz < 2 || q.nx > kMaxNx || q.ny > kMaxNy || q.nz > kMaxNz) return false;
    if ((int64_t)q.nx * q.ny * q.nz > ((int64_t)1 << 28)) return false;
    if (q.nspecies < 1 || q.nspecies > cfg.max_species) return false;
    if (!std::isfinite(q.dt) || q.nsteps < 1) return false;
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(q.b0[k])) return false;
    for (int s = 0; s < q.nspecies; ++s) {
        if (!(q.qm[s] != 0.0) || !std::isfinite(q.qm[s]) || !std::isfinite(q.q[s])) return false;
        const ohpic_species_init &p = q.species[s];
        if (!(p.ppc >= 0.0) || !std::isfinite(p.ppc) || !std::isfinite(p.vth)) return false;
    }
    return true;
}

// Counts, segments and byte footprint of a request (host-side draws only).
bool plan_run(const ohpic_serve_config &cfg, const ohpic_run_request &q, Run &r)
{
    if (!request_ok(cfg, q) || !serve_geom(cfg, q.nx, q.ny, q.nz, r.g)) return false;
    r.req = q;
    r.nsp = q.nspecies;
    DrawSpec d;
    d.precision = OHPIC_FP32;
    d.n[0] = q.nx; d.n[1] = q.ny; d.n[2] = q.nz;
    d.initstate = q.seed_state;
    d.initseq = q.seed_seq;
    d.nspecies = q.nspecies;
    d.spi = q.species;
    d.counts_only = true;
    if (draw_particles(d, r.count, nullptr) != OHPIC_OK) return false;
    int64_t off = 0;
    r.total = 0;
    r.items = 0;
    for (int s = 0; s < r.nsp; ++s) {
        r.seg[s] = off;
        off += (r.count[s] + kSegAlign - 1) / kSegAlign * kSegAlign;
        r.total += r.count[s];
        r.items += r.g.ntile;
    }
    if (r.total >= ((int64_t)1 << 31)) return false;
    r.slots = std::max<int64_t>(off, kSegAlign);
    r.out_doubles = (q.keep_fields ? 5 * r.g.ncell : 0) + (q.keep_particles ? 6 * r.total : 0);
    r.bytes = run_layout(r.slots, r.nsp, r.g.ntile, q.keep_particles != 0, r.out_doubles).total;
    ohpic_config k;
    ohpic_config_default(&k);
    for (int s = 0; s < r.nsp; ++s) {
        k.qm[s] = q.qm[s];
        k.q[s] = q.q[s];
    }
    for (int c = 0; c < 3; ++c) k.b0[c] = q.b0[c];
    for (int s = 0; s < r.nsp; ++s) species_consts(k, s, q.dt, r.sc[s]);
    return true;
}

}  // namespace

extern "C" {

void ohpic_serve_config_default(ohpic_serve_config *cfg)
{
    if (!cfg) return;
    memset(cfg, 0, sizeof(*cfg));
    cfg->max_active = kMaxServeRuns;
    cfg->slots_per_pool = 16;
    cfg->sort_every = 8;
    cfg->sort_lead = 4;
    cfg->use_graphs = 1;
    cfg->weights = OHPIC_WEIGHTS_REFERENCE;
    cfg->halo = 1;
    cfg->deposit = OHPIC_DEPOSIT_LANES;
    cfg->max_species = 2;
}

void ohpic_run_request_default(ohpic_run_request *req)
{
    if (!req) return;
    memset(req, 0, sizeof(*req));
    req->nx = req->ny = req->nz = 16;
    req->nspecies = 2;
    req->dt = 0.1;
    req->qm[0] = -1.0;
    req->qm[1] = 0.01;
    for (int s = 0; s < OHPIC_MAX_SPECIES; ++s)
        for (int k = 0; k < 3; ++k) {
            req->species[s].lo[k] = 0.0;
            req->species[s].hi[k] = 1e30;
        }
    req->seed_state = 42;
    req->seed_seq = 52;
    req->nsteps = 1;
}

static bool normalise(const ohpic_serve_config *in, ohpic_serve_config &c)
{
    c = *in;
    if (c.max_active <= 0 || c.max_active > kMaxServeRuns) c.max_active = kMaxServeRuns;
    if (c.slots_per_pool <= 0) c.slots_per_pool = 16;
    if (c.slots_per_pool > 256) return false;
    if (c.sort_every < 0) return false;
    if (c.sort_every == 0) c.sort_every = 8;
    if (c.sort_lead < 0 || c.sort_lead > 4096) return false;
    if (c.halo <= 0) c.halo = 1;
    if (c.halo > kMaxHalo) return false;
    if (c.tile < 0 || c.tile > 64 || c.tile_x < 0 || c.tile_x > 64) return false;
    if (c.max_species <= 0) c.max_species = 2;
    if (c.max_species > OHPIC_MAX_SPECIES) return false;
    if (c.lane_particles == 0) c.lane_particles = 4;
    if (c.lane_particles != 2 && c.lane_particles != 4) return false;
    if (c.weights != OHPIC_WEIGHTS_REFERENCE && c.weights != OHPIC_WEIGHTS_STANDARD) return false;
    if (c.deposit < OHPIC_DEPOSIT_RUNS || c.deposit > OHPIC_DEPOSIT_LANES) return false;
    return true;
}

int64_t ohpic_serve_footprint(const ohpic_serve_config *cfg, const ohpic_run_request *req)
{
    if (!cfg || !req) return -1;
    ohpic_serve_config c;
    if (!normalise(cfg, c)) return -1;
    Run r;
    if (!plan_run(c, *req, r)) return -1;
    return r.bytes;
}

int ohpic_serve_create(const ohpic_serve_config *cfg, ohpic_server **out)
{
    if (!cfg || !out) return OHPIC_ERR_INVALID;
    *out = nullptr;
    ohpic_serve_config c;
    if (!normalise(cfg, c)) return OHPIC_ERR_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || c.device < 0 || c.device >= ndev) {
        cudaGetLastError();
        return OHPIC_ERR_CUDA;
    }
    cudaSetDevice(c.device);
    std::unique_ptr<Server> s(new (std::nothrow) Server());
    if (!s) return OHPIC_ERR_OOM;
    s->dev = c.device;
    s->t0 = std::chrono::steady_clock::now();
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, c.device);
    if (c.hbm_budget <= 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        c.hbm_budget = (int64_t)(0.6 * (double)fr);
    }
    s->cfg = c;
    if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) return OHPIC_ERR_CUDA;
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = c.device;
    if (cudaMemPoolCreate(&s->mempool, &props) != cudaSuccess) {
        cudaStreamDestroy(s->st);
        cudaGetLastError();
        return OHPIC_ERR_CUDA;
    }
    uint64_t keep = (uint64_t)c.hbm_budget;
    cudaMemPoolSetAttribute(s->mempool, cudaMemPoolAttrReleaseThreshold, &keep);
    s->stage_bytes = (size_t)4 << 20;
    bool ok = salloc(s.get(), &s->d_runs, (int64_t)sizeof(RunDesc) * kMaxServeRuns) &&
              salloc(s.get(), &s->d_item_end, 8 * (int64_t)kMaxServeRuns) &&
              salloc(s.get(), &s->d_segs, (int64_t)sizeof(SortSeg) * kMaxSortSegs) &&
              salloc(s.get(), &s->d_chunk_end, 4 * (int64_t)kMaxSortSegs) &&
              salloc(s.get(), &s->d_cursor, 256) && salloc(s.get(), &s->d_nums, 256);
    for (int i = 0; ok && i < kStageSlots; ++i) {
        ok = cudaMallocHost((void **)&s->h_stage[i], s->stage_bytes) == cudaSuccess &&
             cudaEventCreateWithFlags(&s->stage_ev[i], cudaEventDisableTiming) == cudaSuccess;
    }
    for (int i = 0; ok && i < kDepth; ++i)
        ok = cudaEventCreateWithFlags(&s->tick_ev[i], cudaEventDisableTiming) == cudaSuccess;
    if (ok) ok = cudaStreamSynchronize(s->st) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        Server *raw = s.release();
        raw->worker = std::thread();
        ohpic_serve_destroy(raw);
        return OHPIC_ERR_OOM;
    }
    s->stats.budget = c.hbm_budget;
    Server *raw = s.release();
    raw->worker = std::thread(worker_main, raw);
    *out = raw;
    return OHPIC_OK;
}

int ohpic_serve_destroy(ohpic_server *s)
{
    if (!s) return OHPIC_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->dev);
    if (s->st) cudaStreamSynchronize(s->st);
    for (Run *r : s->retiring)
        if (r->ev) cudaEventDestroy(r->ev);
    for (auto &kv : s->runs)
        if (kv.second->mem) sfree(s, kv.second->mem);
    for (auto &P : s->pools) destroy_pool(s, P.get());
    for (void *p : {(void *)s->d_count, (void *)s->d_start, (void *)s->d_cur32, (void *)s->d_scan_tmp,
                    (void *)s->d_runs, (void *)s->d_item_end, (void *)s->d_segs, (void *)s->d_chunk_end,
                    (void *)s->d_cursor, (void *)s->d_nums})
        sfree(s, p);
    if (s->g_tick) cudaGraphExecDestroy(s->g_tick);
    if (s->g_sort) cudaGraphExecDestroy(s->g_sort);
    if (s->st) cudaStreamSynchronize(s->st);
    for (int i = 0; i < kStageSlots; ++i) {
        if (s->h_stage[i]) cudaFreeHost(s->h_stage[i]);
        if (s->stage_ev[i]) cudaEventDestroy(s->stage_ev[i]);
    }
    for (int i = 0; i < kDepth; ++i)
        if (s->tick_ev[i]) cudaEventDestroy(s->tick_ev[i]);
    if (s->mempool) cudaMemPoolDestroy(s->mempool);
    if (s->st) cudaStreamDestroy(s->st);
    cudaGetLastError();
    delete s;
    return OHPIC_OK;
}

int ohpic_serve_submit(ohpic_server *s, const ohpic_run_request *req, int64_t *id)
{
    if (!s || !req) return OHPIC_ERR_INVALID;
    std::unique_ptr<Run> r(new (std::nothrow) Run());
    if (!r) return OHPIC_ERR_OOM;
    if (!plan_run(s->cfg, *req, *r)) {
        s->set_err("submit: invalid request (grid 2..2048 x 2048 x 1024, 1..max_species species, finite "
                   "non-zero qm, nsteps >= 1) or a staged tile box too large for shared memory");
        return OHPIC_ERR_INVALID;
    }
    if (r->bytes + pool_bytes(r->g, s->cfg.slots_per_pool, s->cfg.max_species) > s->cfg.hbm_budget)
        return OHPIC_ERR_CAPACITY;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->dead) return OHPIC_ERR_CUDA;
    r->id = s->next_id++;
    r->t_submit = s->now();
    if (id) *id = r->id;
    Run *raw = r.get();
    s->runs[raw->id] = std::move(r);
    s->incoming.push_back(raw);
    s->outstanding += 1;
    s->stats.submitted += 1;
    s->cv_work.notify_all();
    return OHPIC_OK;
}

int ohpic_serve_poll(ohpic_server *s, int64_t *ids, int32_t cap, int32_t *n)
{
    if (!s || !n || cap < 0 || (cap > 0 && !ids)) return OHPIC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    int32_t k = 0;
    while (k < cap && !s->completed.empty()) {
        ids[k++] = s->completed.front();
        s->completed.pop_front();
    }
    *n = k;
    return OHPIC_OK;
}

int ohpic_serve_wait(ohpic_server *s, double timeout_s)
{
    if (!s) return OHPIC_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto pred = [&] { return s->outstanding == 0 || s->dead; };
    if (timeout_s > 0) {
        if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred)) return OHPIC_ERR_TIMEOUT;
    } else {
        s->cv_done.wait(lk, pred);
    }
    return s->dead ? OHPIC_ERR_CUDA : OHPIC_OK;
}

int ohpic_serve_result(ohpic_server *s, int64_t id, ohpic_run_result *res, double *fields, double *particles)
{
    if (!s || !res) return OHPIC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->runs.find(id);
    if (it == s->runs.end()) return OHPIC_ERR_INVALID;
    const Run &r = *it->second;
    memset(res, 0, sizeof(*res));
    res->id = r.id;
    res->status = r.status;
    res->done = r.done ? 1 : 0;
    res->steps = r.steps;
    res->particles = r.total;
    res->submit_s = r.t_submit;
    res->admit_s = r.t_admit;
    res->finish_s = r.t_finish;
    if (r.done) res->diag = r.diag_out;
    if (r.done && fields && !r.fields.empty()) memcpy(fields, r.fields.data(), r.fields.size() * 8);
    if (r.done && particles && !r.parts.empty()) memcpy(particles, r.parts.data(), r.parts.size() * 8);
    return OHPIC_OK;
}

int ohpic_serve_release(ohpic_server *s, int64_t id)
{
    if (!s) return OHPIC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->runs.find(id);
    if (it == s->runs.end() || !it->second->done) return OHPIC_ERR_INVALID;
    s->runs.erase(it);
    return OHPIC_OK;
}

int ohpic_serve_stats_get(ohpic_server *s, ohpic_serve_stats *st)
{
    if (!s || !st) return OHPIC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *st = s->stats;
    return OHPIC_OK;
}

int ohpic_serve_last_error(ohpic_server *s, char *buf, size_t len)
{
    if (!s || !buf || len == 0) return OHPIC_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    const size_t n = std::min(len - 1, s->err.size());
    memcpy(buf, s->err.data(), n);
    buf[n] = '\0';
    return OHPIC_OK;
}

}  // extern "C"
