// init.cu -- device-side initial conditions with the reference injector's streams.
//
// Reference: the driver seeds one PCG32 stream with (42, 52) and advances it by
// rank*1e8 (src/ohhelppic3d.f90:111-112); each species then draws once for
// random_fix (src/radom/random_generator.f90:45-58) and 7 times per particle:
// x, y, z as rand()*(upper-lower)+lower (position_random_uniform_distribution.f90:38-41)
// and 4 draws for the 3-D Maxwellian (velocity_maxwell_distribution3d.f90:41-56,
// with sigma = vth, no factor 2), clipped to +-6 sigma.
//
// Because every particle consumes exactly 7 draws, thread i jumps its copy of
// the stream ahead by 7*i (O(log i) affine-map squaring) and needs no
// communication.  Positions are bit-identical to a host injector using the same
// streams (exact uniform draws, one rounded multiply and one rounded add);
// velocities use the device's log/sqrt/cos/sin and may differ from a host libm in
// the last bit.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

constexpr uint64_t kPcgMult = 6364136223846793005ULL;
constexpr double kRefPi = 3.14159265358979;   // src/utils/science_constants.f90:4

struct Pcg {
    uint64_t state, inc;
};

__host__ __device__ inline uint32_t pcg_next(Pcg &r)
{
    const uint64_t old = r.state;
    r.state = old * kPcgMult + r.inc;
    const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}

// Jump ahead by delta steps: compose s -> a*s + c with itself by squaring.
__host__ __device__ inline void pcg_advance(Pcg &r, uint64_t delta)
{
    uint64_t am = 1u, ap = 0u, cm = kPcgMult, cp = r.inc;
    while (delta) {
        if (delta & 1u) {
            am *= cm;
            ap = ap * cm + cp;
        }
        cp = (cm + 1u) * cp;
        cm *= cm;
        delta >>= 1u;
    }
    r.state = am * r.state + ap;
}

__host__ __device__ inline Pcg pcg_seed(uint64_t initstate, uint64_t initseq)
{
    Pcg r{0u, (initseq << 1u) | 1u};
    r.state = r.state * kPcgMult + r.inc;
    r.state += initstate;
    r.state = r.state * kPcgMult + r.inc;
    return r;
}

// pcg32_random_double_r: a 32-bit draw times 2^-32 (exact).
__host__ __device__ inline double pcg_double(Pcg &r) { return (double)pcg_next(r) * 2.3283064365386963e-10; }

struct InitArgs {
    Pcg base;          // stream position of the species' first particle draw
    int64_t n;
    int64_t dst;       // absolute slot of particle 0
    double lo[3], hi[3];
    double vth;
    double drift[3];
    int nx, ny, nz;
};

__device__ inline void sample(const InitArgs &a, int64_t i, double pos[3], double vel[3])
{
    Pcg r = a.base;
    pcg_advance(r, (uint64_t)(7 * i));
    for (int d = 0; d < 3; ++d) pos[d] = __dadd_rn(__dmul_rn(pcg_double(r), __dsub_rn(a.hi[d], a.lo[d])), a.lo[d]);
    const double r1 = pcg_double(r), r2 = pcg_double(r), r3 = pcg_double(r), r4 = pcg_double(r);
    const double sigma = a.vth;
    const double m1 = sigma * sqrt(-2.0 * log(r1)), m3 = sigma * sqrt(-2.0 * log(r3));
    double v[3] = {m1 * cos(2.0 * kRefPi * r2), m1 * sin(2.0 * kRefPi * r2), m3 * sin(2.0 * kRefPi * r4)};
    for (int d = 0; d < 3; ++d) {
        double c = v[d] < sigma * 6 ? v[d] : sigma * 6;
        c = -sigma * 6 > c ? -sigma * 6 : c;
        vel[d] = c + a.drift[d];
    }
}

__global__ void k_init_f64(InitArgs a, PartF64 p, uint32_t *ids)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        double pos[3], vel[3];
        sample(a, i, pos, vel);
        const int64_t o = a.dst + i;
        p.x[o] = pos[0]; p.y[o] = pos[1]; p.z[o] = pos[2];
        p.vx[o] = vel[0]; p.vy[o] = vel[1]; p.vz[o] = vel[2];
        if (ids) ids[o] = (uint32_t)i;
    }
}

__device__ inline void split(double x, int n, int &c, float &o)
{
    int k = (int)floor(x);
    float f = (float)(x - (double)k);
    if (f >= 1.f) { f = 0.f; ++k; }
    if (k >= n) k -= n;
    if (k < 0) k += n;
    c = k;
    o = f;
}

__global__ void k_init_f32(InitArgs a, PartF32 p, uint32_t *ids)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n; i += (int64_t)gridDim.x * blockDim.x) {
        double pos[3], vel[3];
        sample(a, i, pos, vel);
        int cx, cy, cz;
        float ox, oy, oz;
        split(pos[0], a.nx, cx, ox);
        split(pos[1], a.ny, cy, oy);
        split(pos[2], a.nz, cz, oz);
        const int64_t o = a.dst + i;
        p.cell[o] = pack_cell(cx, cy, cz);
        p.ox[o] = ox; p.oy[o] = oy; p.oz[o] = oz;
        p.vx[o] = (float)vel[0]; p.vy[o] = (float)vel[1]; p.vz[o] = (float)vel[2];
        if (ids) ids[o] = (uint32_t)i;
    }
}

}  // namespace

int draw_particles(const DrawSpec &d, int64_t *counts, std::string *err)
{
    Pcg rng = pcg_seed(d.initstate, d.initseq);
    pcg_advance(rng, d.advance);
    for (int s = 0; s < d.nspecies; ++s) {
        const ohpic_species_init &p = d.spi[s];
        InitArgs a;
        double volume = 1.0;
        for (int k = 0; k < 3; ++k) {
            a.hi[k] = p.hi[k] < (double)d.n[k] ? p.hi[k] : (double)d.n[k];
            a.lo[k] = p.lo[k] > 0.0 ? p.lo[k] : 0.0;
            const double w = a.hi[k] - a.lo[k];
            volume *= w > 0.0 ? w : 0.0;
            a.drift[k] = p.drift[k];
        }
        // random_fix(ppc * volume): one draw decides whether the fraction rounds up.
        const double value = p.ppc * volume;
        const int64_t fixed = (int64_t)value;
        const int64_t count = pcg_double(rng) <= value - (double)fixed ? fixed + 1 : fixed;
        if (d.cap && count > d.cap[s]) {
            if (err) *err = "init: species " + std::to_string(s) + " needs " + std::to_string(count) + " > capacity";
            return OHPIC_ERR_CAPACITY;
        }
        a.base = rng;
        a.n = count;
        a.dst = d.seg ? d.seg[s] : 0;
        a.vth = p.vth;
        a.nx = d.n[0]; a.ny = d.n[1]; a.nz = d.n[2];
        if (!d.counts_only && count > 0) {
            int64_t blocks = (count + 255) / 256;
            if (blocks > 152 * 64) blocks = 152 * 64;
            if (d.precision == OHPIC_FP64)
                k_init_f64<<<(unsigned)blocks, 256, 0, d.stream>>>(a, d.p64, d.ids);
            else
                k_init_f32<<<(unsigned)blocks, 256, 0, d.stream>>>(a, d.p32, d.ids);
            if (d.launches) ++*d.launches;
        }
        pcg_advance(rng, (uint64_t)(7 * count));
        if (counts) counts[s] = count;
    }
    return OHPIC_OK;
}

int init_particles(ohpic_ctx *c, uint64_t initstate, uint64_t initseq, uint64_t advance,
                   const ohpic_species_init *spi, int64_t *counts)
{
    DrawSpec d;
    d.stream = c->stream;
    d.precision = c->cfg.precision;
    d.n[0] = c->g.nx; d.n[1] = c->g.ny; d.n[2] = c->g.nz;
    d.initstate = initstate;
    d.initseq = initseq;
    d.advance = advance;
    d.nspecies = c->cfg.nspecies;
    d.spi = spi;
    d.seg = c->seg;
    d.cap = c->cap;
    materialize_records(c);
    d.p64 = c->p64[c->cur];
    d.p32 = c->p32[c->cur];
    d.ids = c->ids[c->cur];
    d.launches = &c->launches;
    int64_t cnt[OHPIC_MAX_SPECIES] = {0};
    const int rc = draw_particles(d, cnt, &c->err);
    if (rc != OHPIC_OK) return rc;
    for (int s = 0; s < c->cfg.nspecies; ++s) {
        c->count[s] = cnt[s];
        if (counts) counts[s] = cnt[s];
    }
    c->sorted = false;
    c->rho_valid = false;
    c->kin_valid = false;
    return OHPIC_OK;
}

}  // namespace ohpic
