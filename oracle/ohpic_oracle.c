/*
 * ohpic_oracle.c -- CPU restatement of ohhelppic3d's per-timestep particle path.
 *
 * TEST INFRASTRUCTURE ONLY (the correctness checker and the timed CPU baseline);
 * see ohpic_oracle.h for the list of reference files each part follows and for
 * the documented deviations D1-D7.  Build with -ffp-contract=off so that every
 * multiply and add rounds separately, as the Fortran source does.
 *
 * With one thread every loop runs in the reference's order (species, then
 * particle index).  With more threads the particle loops are split into
 * contiguous ranges and the deposit uses one private rho per thread, reduced
 * in thread order; the result then differs from the one-thread result only by
 * the summation order of rho.
 */
#include "ohpic_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* The reference's pi literal (src/utils/science_constants.f90:4), used by the
 * Green's function (poisson_solver3d.f90:114,116) and the Maxwellian sampler. */
static const double REF_PI = 3.14159265358979;
/* Full-precision 2*pi for the FFT twiddles (FFTW's own twiddles are exact). */
static const double TWO_PI_EXACT = 6.283185307179586476925286766559;

/* ------------------------------------------------------------------------ */
/* PCG32: 64-bit LCG state, odd increment selects the stream, XSH-RR output.  */
/* Published PCG algorithm (O'Neill 2014); the reference binds it through     */
/* src/radom/pcg/pcg64.f90:10-32 and pcg_generator.f90:29-41.                  */
/* ------------------------------------------------------------------------ */
static const uint64_t PCG_MULT = 6364136223846793005ULL;

static inline void pcg_step(orc_pcg32 *rng) { rng->state = rng->state * PCG_MULT + rng->inc; }

void orc_pcg32_srandom(orc_pcg32 *rng, uint64_t initstate, uint64_t initseq)
{
    rng->state = 0u;
    rng->inc = (initseq << 1u) | 1u;
    pcg_step(rng);
    rng->state += initstate;
    pcg_step(rng);
}

uint32_t orc_pcg32_random(orc_pcg32 *rng)
{
    uint64_t old = rng->state;
    pcg_step(rng);
    uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
}

/* Jump ahead by delta steps in O(log delta): compose the affine map
 * s -> a*s + c with itself by repeated squaring (Brown, "Random number
 * generation with arbitrary strides", 1994).  delta is taken modulo 2^64, so a
 * "negative" delta rewinds. */
void orc_pcg32_advance(orc_pcg32 *rng, uint64_t delta)
{
    /* total: the map for the bits of delta consumed so far; step: the map for
     * 2^bit steps, squared once per bit (a*(a*s+c)+c = a^2 s + (a+1) c). */
    uint64_t total_a = 1u, total_c = 0u;
    uint64_t step_a = PCG_MULT, step_c = rng->inc;
    for (; delta; delta >>= 1u) {
        if (delta & 1u) {
            total_a = total_a * step_a;
            total_c = total_c * step_a + step_c;
        }
        step_c = step_c * (step_a + 1u);
        step_a = step_a * step_a;
    }
    rng->state = total_a * rng->state + total_c;
}

/* pcg32_random_double_r: a 32-bit draw scaled by 2^-32 (lib/pcg-c/src/pcg32_double.c:60-63). */
double orc_pcg32_double(orc_pcg32 *rng) { return ldexp((double)orc_pcg32_random(rng), -32); }

void orc_pcg32_fill(uint64_t initstate, uint64_t initseq, uint64_t advance, uint32_t *out,
                    int64_t n)
{
    orc_pcg32 r;
    orc_pcg32_srandom(&r, initstate, initseq);
    orc_pcg32_advance(&r, advance);
    for (int64_t i = 0; i < n; ++i) out[i] = orc_pcg32_random(&r);
}

/* ------------------------------------------------------------------------ */
/* Simulation state                                                           */
/* ------------------------------------------------------------------------ */
struct orc_sim {
    orc_config cfg;
    int nthreads;
    int64_t ncell;
    int64_t np[ORC_MAX_SPECIES];
    double *x[ORC_MAX_SPECIES], *y[ORC_MAX_SPECIES], *z[ORC_MAX_SPECIES];
    double *vx[ORC_MAX_SPECIES], *vy[ORC_MAX_SPECIES], *vz[ORC_MAX_SPECIES];
    double *rho;   /* nx*ny*nz after the ghost fold */
    double *phi;   /* nx*ny*nz */
    double *ex, *ey, *ez;
    int64_t crossings[3];
};

static inline int64_t nidx(const orc_sim *s, int i, int j, int k)
{
    return (int64_t)i + (int64_t)s->cfg.nx * ((int64_t)j + (int64_t)s->cfg.ny * k);
}

orc_sim *orc_create(const orc_config *cfg)
{
    if (cfg->nx <= 0 || cfg->ny <= 0 || cfg->nz <= 0) return NULL;
    if (cfg->nspecies < 1 || cfg->nspecies > ORC_MAX_SPECIES) return NULL;
    orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
    if (!s) return NULL;
    s->cfg = *cfg;
    s->nthreads = 1;
    s->ncell = (int64_t)cfg->nx * cfg->ny * cfg->nz;
    for (int sp = 0; sp < cfg->nspecies; ++sp) {
        int64_t cap = cfg->capacity[sp] > 0 ? cfg->capacity[sp] : 1;
        s->x[sp] = (double *)malloc(sizeof(double) * cap);
        s->y[sp] = (double *)malloc(sizeof(double) * cap);
        s->z[sp] = (double *)malloc(sizeof(double) * cap);
        s->vx[sp] = (double *)malloc(sizeof(double) * cap);
        s->vy[sp] = (double *)malloc(sizeof(double) * cap);
        s->vz[sp] = (double *)malloc(sizeof(double) * cap);
        if (!s->x[sp] || !s->y[sp] || !s->z[sp] || !s->vx[sp] || !s->vy[sp] || !s->vz[sp]) {
            orc_destroy(s);
            return NULL;
        }
    }
    s->rho = (double *)calloc(s->ncell, sizeof(double));
    s->phi = (double *)calloc(s->ncell, sizeof(double));
    s->ex = (double *)calloc(s->ncell, sizeof(double));
    s->ey = (double *)calloc(s->ncell, sizeof(double));
    s->ez = (double *)calloc(s->ncell, sizeof(double));
    if (!s->rho || !s->phi || !s->ex || !s->ey || !s->ez) {
        orc_destroy(s);
        return NULL;
    }
    return s;
}

void orc_destroy(orc_sim *s)
{
    if (!s) return;
    for (int sp = 0; sp < ORC_MAX_SPECIES; ++sp) {
        free(s->x[sp]); free(s->y[sp]); free(s->z[sp]);
        free(s->vx[sp]); free(s->vy[sp]); free(s->vz[sp]);
    }
    free(s->rho); free(s->phi); free(s->ex); free(s->ey); free(s->ez);
    free(s);
}

void orc_set_threads(orc_sim *s, int nthreads) { s->nthreads = nthreads < 1 ? 1 : nthreads; }

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int64_t orc_count(const orc_sim *s, int sp) { return (sp >= 0 && sp < s->cfg.nspecies) ? s->np[sp] : -1; }

int orc_set_particles(orc_sim *s, int sp, const double *x, const double *y, const double *z,
                      const double *vx, const double *vy, const double *vz, int64_t n)
{
    if (sp < 0 || sp >= s->cfg.nspecies || n < 0 || n > s->cfg.capacity[sp]) return -1;
    memcpy(s->x[sp], x, sizeof(double) * n);
    memcpy(s->y[sp], y, sizeof(double) * n);
    memcpy(s->z[sp], z, sizeof(double) * n);
    memcpy(s->vx[sp], vx, sizeof(double) * n);
    memcpy(s->vy[sp], vy, sizeof(double) * n);
    memcpy(s->vz[sp], vz, sizeof(double) * n);
    s->np[sp] = n;
    return 0;
}

int64_t orc_get_particles(const orc_sim *s, int sp, double *x, double *y, double *z, double *vx,
                          double *vy, double *vz)
{
    if (sp < 0 || sp >= s->cfg.nspecies) return -1;
    int64_t n = s->np[sp];
    if (x) memcpy(x, s->x[sp], sizeof(double) * n);
    if (y) memcpy(y, s->y[sp], sizeof(double) * n);
    if (z) memcpy(z, s->z[sp], sizeof(double) * n);
    if (vx) memcpy(vx, s->vx[sp], sizeof(double) * n);
    if (vy) memcpy(vy, s->vy[sp], sizeof(double) * n);
    if (vz) memcpy(vz, s->vz[sp], sizeof(double) * n);
    return n;
}

static double *field_ptr(const orc_sim *s, int which)
{
    switch (which) {
    case ORC_RHO: return s->rho;
    case ORC_PHI: return s->phi;
    case ORC_EX: return s->ex;
    case ORC_EY: return s->ey;
    case ORC_EZ: return s->ez;
    default: return NULL;
    }
}

void orc_get_field(const orc_sim *s, int which, double *out)
{
    double *f = field_ptr(s, which);
    if (f) memcpy(out, f, sizeof(double) * s->ncell);
}

void orc_set_field(orc_sim *s, int which, const double *in)
{
    double *f = field_ptr(s, which);
    if (f) memcpy(f, in, sizeof(double) * s->ncell);
}

/* ------------------------------------------------------------------------ */
/* Initial conditions                                                         */
/* ------------------------------------------------------------------------ */

/* random_fix (src/radom/random_generator.f90:45-58): one draw decides whether
 * the fractional part rounds up. */
static int64_t random_fix(orc_pcg32 *rng, double value)
{
    int64_t fixed = (int64_t)value;
    if (orc_pcg32_double(rng) <= value - (double)fixed) return fixed + 1;
    return fixed;
}

/* One particle: x, y, z uniform draws (position_random_uniform_distribution.f90:38-41,
 * rand()*(upper-lower)+lower), then the 4-draw Maxwellian
 * (velocity_maxwell_distribution3d.f90:41-56) with sigma = vth (D3). */
static void sample_particle(orc_pcg32 *rng, const double lo[3], const double hi[3], double vth,
                            const double drift[3], double pos[3], double vel[3])
{
    for (int d = 0; d < 3; ++d) pos[d] = orc_pcg32_double(rng) * (hi[d] - lo[d]) + lo[d];
    double r1 = orc_pcg32_double(rng);
    double r2 = orc_pcg32_double(rng);
    double r3 = orc_pcg32_double(rng);
    double r4 = orc_pcg32_double(rng);
    double sigma = vth;
    double v[3];
    v[0] = sigma * sqrt(-2.0 * log(r1)) * cos(2.0 * REF_PI * r2);
    v[1] = sigma * sqrt(-2.0 * log(r1)) * sin(2.0 * REF_PI * r2);
    v[2] = sigma * sqrt(-2.0 * log(r3)) * sin(2.0 * REF_PI * r4);
    for (int d = 0; d < 3; ++d) {
        double c = v[d] < sigma * 6 ? v[d] : sigma * 6;       /* min(ret, sigma*6) */
        c = -sigma * 6 > c ? -sigma * 6 : c;                 /* max(-sigma*6, ...) */
        vel[d] = c + drift[d];
    }
}

int orc_init_particles(orc_sim *s, uint64_t initstate, uint64_t initseq, uint64_t rank_advance,
                       const orc_species_init *spi)
{
    orc_pcg32 rng;
    orc_pcg32_srandom(&rng, initstate, initseq);   /* src/ohhelppic3d.f90:111 */
    orc_pcg32_advance(&rng, rank_advance);         /* src/ohhelppic3d.f90:112 */
    const int n[3] = {s->cfg.nx, s->cfg.ny, s->cfg.nz};
    for (int sp = 0; sp < s->cfg.nspecies; ++sp) {
        const orc_species_init *p = &spi[sp];
        double lo[3], hi[3], volume = 1.0;
        for (int d = 0; d < 3; ++d) {
            /* min/max against the (single) subdomain [0, n]. */
            hi[d] = p->hi[d] < (double)n[d] ? p->hi[d] : (double)n[d];
            lo[d] = p->lo[d] > 0.0 ? p->lo[d] : 0.0;
            volume *= (hi[d] - lo[d]) > 0.0 ? (hi[d] - lo[d]) : 0.0;
        }
        int64_t count = random_fix(&rng, p->ppc * volume);
        if (count > s->cfg.capacity[sp]) return -1;
        /* Every particle consumes exactly 7 draws, so thread ranges can start
         * from a jump-ahead copy of the stream and stay bit-identical to the
         * sequential loop. */
        orc_pcg32 base = rng;
        double *X = s->x[sp], *Y = s->y[sp], *Z = s->z[sp];
        double *VX = s->vx[sp], *VY = s->vy[sp], *VZ = s->vz[sp];
#pragma omp parallel num_threads(s->nthreads)
        {
            int nt = 1, tid = 0;
#ifdef _OPENMP
            nt = omp_get_num_threads();
            tid = omp_get_thread_num();
#endif
            int64_t a = count * tid / nt, b = count * (tid + 1) / nt;
            orc_pcg32 r = base;
            orc_pcg32_advance(&r, (uint64_t)(7 * a));
            for (int64_t i = a; i < b; ++i) {
                double pos[3], vel[3];
                sample_particle(&r, lo, hi, p->vth, p->drift, pos, vel);
                X[i] = pos[0]; Y[i] = pos[1]; Z[i] = pos[2];
                VX[i] = vel[0]; VY[i] = vel[1]; VZ[i] = vel[2];
            }
        }
        orc_pcg32_advance(&rng, (uint64_t)(7 * count));
        s->np[sp] = count;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* CIC weights (D1)                                                           */
/* ------------------------------------------------------------------------ */
/* w[0] is the weight of node floor(x), w[1] of node floor(x)+1.  The reference
 * assigns rxyz(1,:) = r, rxyz(2,:) = 1-r (linear_scatter.f90:41-42,
 * linear_interpolator.f90:54-57). */
static inline void cic_weights(int convention, double r, double w[2])
{
    if (convention == ORC_WEIGHTS_REFERENCE) {
        w[0] = r;
        w[1] = 1.0 - r;
    } else {
        w[0] = 1.0 - r;
        w[1] = r;
    }
}

/* ------------------------------------------------------------------------ */
/* Deposit: src/scatter/linear_scatter.f90:32-53 into rho with a ghost node    */
/* at n on every axis, then the periodic fold of the ghost into node 0 (D5).   */
/* ------------------------------------------------------------------------ */
static void deposit_range(const orc_sim *s, int sp, int64_t a, int64_t b, double *g)
{
    const int gx = s->cfg.nx + 1, gy = s->cfg.ny + 1;
    const double amount = s->cfg.q[sp];
    const double *X = s->x[sp], *Y = s->y[sp], *Z = s->z[sp];
    for (int64_t p = a; p < b; ++p) {
        double lx = X[p], ly = Y[p], lz = Z[p];     /* to_local_position: minus 0 */
        double ilx = (double)(int)lx, ily = (double)(int)ly, ilz = (double)(int)lz;
        double wx[2], wy[2], wz[2];
        cic_weights(s->cfg.weights, lx - ilx, wx);
        cic_weights(s->cfg.weights, ly - ily, wy);
        cic_weights(s->cfg.weights, lz - ilz, wz);
        int ix = (int)ilx, iy = (int)ily, iz = (int)ilz;
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    int64_t at = (int64_t)(ix + i) + (int64_t)gx * ((iy + j) + (int64_t)gy * (iz + k));
                    g[at] = g[at] + amount * wx[i] * wy[j] * wz[k];
                }
    }
}

void orc_deposit(orc_sim *s)
{
    const int nx = s->cfg.nx, ny = s->cfg.ny, nz = s->cfg.nz;
    const int gx = nx + 1, gy = ny + 1, gz = nz + 1;
    const int64_t gsize = (int64_t)gx * gy * gz;
    int nt = s->nthreads;
    double *g = (double *)calloc((size_t)gsize * nt, sizeof(double));
    if (!g) return;
    if (nt == 1) {
        for (int sp = 0; sp < s->cfg.nspecies; ++sp) deposit_range(s, sp, 0, s->np[sp], g);
    } else {
#pragma omp parallel num_threads(nt)
        {
            int tid = 0, tn = 1;
#ifdef _OPENMP
            tid = omp_get_thread_num();
            tn = omp_get_num_threads();
#endif
            double *mine = g + gsize * tid;
            for (int sp = 0; sp < s->cfg.nspecies; ++sp) {
                int64_t n = s->np[sp];
                deposit_range(s, sp, n * tid / tn, n * (tid + 1) / tn, mine);
            }
#pragma omp barrier
#pragma omp for schedule(static)
            for (int64_t c = 0; c < gsize; ++c) {
                double acc = g[c];
                for (int t = 1; t < tn; ++t) acc = acc + g[gsize * t + c];
                g[c] = acc;
            }
        }
    }
    /* Periodic fold of the ghost planes, x then y then z. */
    for (int k = 0; k < gz; ++k)
        for (int j = 0; j < gy; ++j) {
            int64_t row = (int64_t)gx * (j + (int64_t)gy * k);
            g[row] = g[row] + g[row + nx];
        }
    for (int k = 0; k < gz; ++k)
        for (int i = 0; i < nx; ++i) {
            int64_t a0 = i + (int64_t)gx * ((int64_t)gy * k);
            int64_t an = i + (int64_t)gx * (ny + (int64_t)gy * k);
            g[a0] = g[a0] + g[an];
        }
    for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
            int64_t a0 = i + (int64_t)gx * j;
            int64_t an = i + (int64_t)gx * (j + (int64_t)gy * nz);
            g[a0] = g[a0] + g[an];
        }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            memcpy(s->rho + nidx(s, 0, j, k), g + (int64_t)gx * (j + (int64_t)gy * k),
                   sizeof(double) * nx);
    free(g);
}

/* ------------------------------------------------------------------------ */
/* FFT: mixed-radix Cooley-Tukey on interleaved complex doubles.              */
/* ------------------------------------------------------------------------ */
typedef struct {
    int n;
    int nf;
    int f[40];
    double *twr, *twi;   /* exp(-2 pi i j / n), j < n */
} fft_plan;

static int fft_plan_init(fft_plan *p, int n)
{
    p->n = n;
    p->nf = 0;
    int m = n;
    for (int r = 2; m > 1;) {
        if (m % r == 0) {
            p->f[p->nf++] = r;
            m /= r;
        } else {
            ++r;
        }
    }
    p->twr = (double *)malloc(sizeof(double) * n);
    p->twi = (double *)malloc(sizeof(double) * n);
    if (!p->twr || !p->twi) return -1;
    for (int j = 0; j < n; ++j) {
        double a = TWO_PI_EXACT * (double)j / (double)n;
        p->twr[j] = cos(a);
        p->twi[j] = -sin(a);
    }
    return 0;
}

static void fft_plan_free(fft_plan *p)
{
    free(p->twr);
    free(p->twi);
}

/* out[k] = sum_j in[j*is] * W^(j*k*step), W = exp(sign 2 pi i / N), for n points. */
static void fft_rec(const double *in, int64_t is, double *out, int n, int step, const fft_plan *P,
                    int fi, int sign, double *tmp)
{
    if (n == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return;
    }
    const int r = P->f[fi], m = n / r, N = P->n;
    for (int q = 0; q < r; ++q) fft_rec(in + 2 * q * is, is * r, out + 2 * q * m, m, step * r, P, fi + 1, sign, tmp);
    double *tr = tmp, *ti = tmp + r;
    for (int k = 0; k < m; ++k) {
        for (int q = 0; q < r; ++q) {
            int e = (int)(((int64_t)q * k * step) % N);
            double wr = P->twr[e], wi = sign < 0 ? P->twi[e] : -P->twi[e];
            double ar = out[2 * (q * m + k)], ai = out[2 * (q * m + k) + 1];
            tr[q] = ar * wr - ai * wi;
            ti[q] = ar * wi + ai * wr;
        }
        for (int sidx = 0; sidx < r; ++sidx) {
            double accr = 0.0, acci = 0.0;
            for (int q = 0; q < r; ++q) {
                int e = (int)(((int64_t)q * sidx * m * step) % N);
                double wr = P->twr[e], wi = sign < 0 ? P->twi[e] : -P->twi[e];
                accr += tr[q] * wr - ti[q] * wi;
                acci += tr[q] * wi + ti[q] * wr;
            }
            out[2 * (k + sidx * m)] = accr;
            out[2 * (k + sidx * m) + 1] = acci;
        }
    }
}

static int max_factor(const fft_plan *p)
{
    int m = 1;
    for (int i = 0; i < p->nf; ++i) m = p->f[i] > m ? p->f[i] : m;
    return m;
}

/* Transform all lines of length n along one axis (element stride es, line
 * origins enumerated by (a, b) with strides sa, sb). */
static void fft_axis(double *data, int n, int64_t es, int na, int64_t sa, int nb, int64_t sb,
                     int sign, int nthreads)
{
    fft_plan P;
    if (fft_plan_init(&P, n) != 0) {
        fft_plan_free(&P);
        return;
    }
    int mf = max_factor(&P);
#pragma omp parallel num_threads(nthreads)
    {
        double *line = (double *)malloc(sizeof(double) * 2 * n);
        double *res = (double *)malloc(sizeof(double) * 2 * n);
        double *tmp = (double *)malloc(sizeof(double) * 2 * mf);
#pragma omp for schedule(static) collapse(2)
        for (int b = 0; b < nb; ++b)
            for (int a = 0; a < na; ++a) {
                double *base = data + 2 * ((int64_t)a * sa + (int64_t)b * sb);
                for (int i = 0; i < n; ++i) {
                    line[2 * i] = base[2 * i * es];
                    line[2 * i + 1] = base[2 * i * es + 1];
                }
                fft_rec(line, 1, res, n, 1, &P, 0, sign, tmp);
                for (int i = 0; i < n; ++i) {
                    base[2 * i * es] = res[2 * i];
                    base[2 * i * es + 1] = res[2 * i + 1];
                }
            }
        free(line);
        free(res);
        free(tmp);
    }
    fft_plan_free(&P);
}

static void fft3d_threads(double *d, int nx, int ny, int nz, int sign, int nt)
{
    fft_axis(d, nx, 1, ny, nx, nz, (int64_t)nx * ny, sign, nt);
    fft_axis(d, ny, nx, nx, 1, nz, (int64_t)nx * ny, sign, nt);
    fft_axis(d, nz, (int64_t)nx * ny, nx, 1, ny, nx, sign, nt);
}

void orc_fft3d(double *data, int nx, int ny, int nz, int sign) { fft3d_threads(data, nx, ny, nz, sign, 1); }

/* ------------------------------------------------------------------------ */
/* Poisson solve (poisson_solver3d.f90:147,184-205 with the periodic wave     */
/* numbers of :104-117 and the 1/(nx*ny*nz) of mpi_fftw3_solver.f90:235).      */
/* ------------------------------------------------------------------------ */
static double wave_number(int k, int n)
{
    if (k <= n / 2) return 2.0 * sin(REF_PI * k / (double)n);
    return 2.0 * sin(REF_PI * (n - k) / (double)n);
}

static double modified_wave_number(int kx, int ky, int kz, int nx, int ny, int nz)
{
    double wx = wave_number(kx, nx), wy = wave_number(ky, ny), wz = wave_number(kz, nz);
    return wx * wx + wy * wy + wz * wz;
}

double orc_green(int kx, int ky, int kz, int nx, int ny, int nz)
{
    if (kx == 0 && ky == 0 && kz == 0) return 0.0;
    return 1.0 / modified_wave_number(kx, ky, kz, nx, ny, nz);
}

void orc_solve(orc_sim *s)
{
    const int nx = s->cfg.nx, ny = s->cfg.ny, nz = s->cfg.nz;
    const int64_t n = s->ncell;
    double *c = (double *)malloc(sizeof(double) * 2 * n);
    if (!c) return;
    for (int64_t i = 0; i < n; ++i) {   /* phi = rho (poisson_solver3d.f90:147) */
        c[2 * i] = s->rho[i];
        c[2 * i + 1] = 0.0;
    }
    fft3d_threads(c, nx, ny, nz, -1, s->nthreads);
#pragma omp parallel for num_threads(s->nthreads) collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int64_t at = nidx(s, i, j, k);
                if (i == 0 && j == 0 && k == 0) {
                    c[2 * at] = 0.0;
                    c[2 * at + 1] = 0.0;
                } else {
                    double wn = modified_wave_number(i, j, k, nx, ny, nz);
                    c[2 * at] = c[2 * at] / wn;
                    c[2 * at + 1] = c[2 * at + 1] / wn;
                }
            }
    fft3d_threads(c, nx, ny, nz, +1, s->nthreads);
    const double norm = (double)nx * (double)ny * (double)nz;
    for (int64_t i = 0; i < n; ++i) s->phi[i] = c[2 * i] / norm;
    free(c);

    /* E: staggered difference then the two-point average of
     * poisson_field_solver.f90:139-144,165-170 (component 1 of phi on every axis, D2):
     * E_d[i] = 0.5 * ((phi[i-e] - phi[i]) + (phi[i] - phi[i+e])). */
    const double *phi = s->phi;
#pragma omp parallel for num_threads(s->nthreads) collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int im = (i + nx - 1) % nx, ip = (i + 1) % nx;
                int jm = (j + ny - 1) % ny, jp = (j + 1) % ny;
                int km = (k + nz - 1) % nz, kp = (k + 1) % nz;
                double p0 = phi[nidx(s, i, j, k)];
                int64_t at = nidx(s, i, j, k);
                s->ex[at] = 0.5 * ((phi[nidx(s, im, j, k)] - p0) + (p0 - phi[nidx(s, ip, j, k)]));
                s->ey[at] = 0.5 * ((phi[nidx(s, i, jm, k)] - p0) + (p0 - phi[nidx(s, i, jp, k)]));
                s->ez[at] = 0.5 * ((phi[nidx(s, i, j, km)] - p0) + (p0 - phi[nidx(s, i, j, kp)]));
            }
}

/* ------------------------------------------------------------------------ */
/* Gather (linear_interpolator.f90:33-67): 8 nodes, i (x) outermost, k (z)    */
/* innermost, ret = ret + v*rx*ry*rz.                                          */
/* ------------------------------------------------------------------------ */
void orc_interp_one(const orc_sim *s, double x, double y, double z, double e[3])
{
    const int nx = s->cfg.nx, ny = s->cfg.ny, nz = s->cfg.nz;
    int ix = (int)x, iy = (int)y, iz = (int)z;
    double wx[2], wy[2], wz[2];
    cic_weights(s->cfg.weights, x - (double)ix, wx);
    cic_weights(s->cfg.weights, y - (double)iy, wy);
    cic_weights(s->cfg.weights, z - (double)iz, wz);
    double r0 = 0.0, r1 = 0.0, r2 = 0.0;
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 2; ++k) {
                int64_t at = nidx(s, (ix + i) % nx, (iy + j) % ny, (iz + k) % nz);
                r0 = r0 + s->ex[at] * wx[i] * wy[j] * wz[k];
                r1 = r1 + s->ey[at] * wx[i] * wy[j] * wz[k];
                r2 = r2 + s->ez[at] * wx[i] * wy[j] * wz[k];
            }
    e[0] = r0;
    e[1] = r1;
    e[2] = r2;
}

/* ------------------------------------------------------------------------ */
/* Boris (particle_mover_boris.f90:37-62) and the position update (:60-62).   */
/* cross(a, b) is the standard component formula (futils m_vector, unpinned). */
/* ------------------------------------------------------------------------ */
static inline void cross3(const double a[3], const double b[3], double c[3])
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

void orc_boris_one(double qm, const double ef[3], const double bf[3], double dt, double pos[3],
                   double vel[3])
{
    double dt2 = dt * 0.5;
    double t[3], s[3], upm[3], upa[3], upp[3], c[3];
    for (int d = 0; d < 3; ++d) t[d] = qm * bf[d] * dt2;
    double tt = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
    for (int d = 0; d < 3; ++d) s[d] = 2.0 * t[d] / (1.0 + tt);
    for (int d = 0; d < 3; ++d) upm[d] = vel[d] + qm * ef[d] * dt2;
    cross3(upm, t, c);
    for (int d = 0; d < 3; ++d) upa[d] = upm[d] + c[d];
    cross3(upa, s, c);
    for (int d = 0; d < 3; ++d) upp[d] = upm[d] + c[d];
    for (int d = 0; d < 3; ++d) vel[d] = upp[d] + qm * ef[d] * dt2;
    for (int d = 0; d < 3; ++d) pos[d] = pos[d] + vel[d] * dt;
}

/* apply_periodic (periodic_particle_boundary.f90:42-53). */
void orc_wrap(int n, double *p)
{
    if (*p < 0) *p = n + *p;
    if (*p >= n) *p = *p - n;
}

void orc_push(orc_sim *s)
{
    const int n[3] = {s->cfg.nx, s->cfg.ny, s->cfg.nz};
    int64_t cx = 0, cy = 0, cz = 0;
    for (int sp = 0; sp < s->cfg.nspecies; ++sp) {
        const double qm = s->cfg.qm[sp];
        double *X = s->x[sp], *Y = s->y[sp], *Z = s->z[sp];
        double *VX = s->vx[sp], *VY = s->vy[sp], *VZ = s->vz[sp];
        const int64_t np = s->np[sp];
#pragma omp parallel for num_threads(s->nthreads) schedule(static) reduction(+ : cx, cy, cz)
        for (int64_t p = 0; p < np; ++p) {
            double e[3], pos[3] = {X[p], Y[p], Z[p]}, vel[3] = {VX[p], VY[p], VZ[p]};
            orc_interp_one(s, pos[0], pos[1], pos[2], e);
            orc_boris_one(qm, e, s->cfg.b0, s->cfg.dt, pos, vel);
            cx += (pos[0] < 0 || pos[0] >= n[0]);
            cy += (pos[1] < 0 || pos[1] >= n[1]);
            cz += (pos[2] < 0 || pos[2] >= n[2]);
            for (int rep = 0; rep < 2; ++rep)   /* ohhelppic3d.f90:353,355 */
                for (int d = 0; d < 3; ++d) orc_wrap(n[d], &pos[d]);
            X[p] = pos[0]; Y[p] = pos[1]; Z[p] = pos[2];
            VX[p] = vel[0]; VY[p] = vel[1]; VZ[p] = vel[2];
        }
    }
    s->crossings[0] = cx;
    s->crossings[1] = cy;
    s->crossings[2] = cz;
}

void orc_step(orc_sim *s, int nsteps)
{
    for (int it = 0; it < nsteps; ++it) {   /* mainstep, ohhelppic3d.f90:311-358 */
        orc_deposit(s);
        orc_solve(s);
        orc_push(s);
    }
}

void orc_diagnostics(orc_sim *s, orc_diag *d)
{
    memset(d, 0, sizeof(*d));
    double qsum = 0.0, fe = 0.0;
    for (int64_t i = 0; i < s->ncell; ++i) {
        qsum += s->rho[i];
        fe += s->ex[i] * s->ex[i] + s->ey[i] * s->ey[i] + s->ez[i] * s->ez[i];
    }
    d->total_charge = qsum;
    d->field_energy = 0.5 * fe;
    double ke = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
    for (int sp = 0; sp < s->cfg.nspecies; ++sp) {
        double m = s->cfg.q[sp] / s->cfg.qm[sp];
        double k2 = 0.0, px = 0.0, py = 0.0, pz = 0.0;
        for (int64_t p = 0; p < s->np[sp]; ++p) {
            k2 += s->vx[sp][p] * s->vx[sp][p] + s->vy[sp][p] * s->vy[sp][p] + s->vz[sp][p] * s->vz[sp][p];
            px += s->vx[sp][p];
            py += s->vy[sp][p];
            pz += s->vz[sp][p];
        }
        ke += 0.5 * m * k2;
        mx += m * px;
        my += m * py;
        mz += m * pz;
        d->count[sp] = s->np[sp];
    }
    d->kinetic_energy = ke;
    d->momentum[0] = mx;
    d->momentum[1] = my;
    d->momentum[2] = mz;
    for (int a = 0; a < 3; ++a) d->crossings[a] = s->crossings[a];
}

/* ------------------------------------------------------------------------ */
/* Bounded-domain field solve (non-periodic kinds).  The restatement follows  */
/* the reference's own algorithm: FFTW's r2r transforms per axis (written     */
/* here as their defining sums), the logical ranges and normalisers of        */
/* mpi_fftw3_solver.f90:151-207, the table and wall terms of                  */
/* poisson_solver3d.f90:56-132 and the solve of :134-207.                      */
/* ------------------------------------------------------------------------ */
enum { R2R_R2HC = 0, R2R_HC2R, R2R_RODFT00, R2R_REDFT00, R2R_RODFT01, R2R_RODFT10, R2R_REDFT01, R2R_REDFT10 };

/* sin and cos of pi * a / b with the integer numerator reduced modulo 2b first
 * (exact pi, like FFTW's own twiddles). */
static double sinpi_frac(int64_t a, int64_t b)
{
    a %= 2 * b;
    if (a < 0) a += 2 * b;
    return sin(TWO_PI_EXACT * 0.5 * (double)a / (double)b);
}
static double cospi_frac(int64_t a, int64_t b)
{
    a %= 2 * b;
    if (a < 0) a += 2 * b;
    return cos(TWO_PI_EXACT * 0.5 * (double)a / (double)b);
}

void orc_r2r_1d(int kind, const double *x, double *y, int N)
{
    switch (kind) {
    case R2R_R2HC:   /* r_k = sum x_j cos(2 pi jk/N), i_k = -sum x_j sin(2 pi jk/N), y[N-k] = i_k */
        for (int k = 0; k <= N / 2; ++k) {
            double re = 0.0, im = 0.0;
            for (int j = 0; j < N; ++j) {
                re += x[j] * cospi_frac(2 * (int64_t)j * k, N);
                im -= x[j] * sinpi_frac(2 * (int64_t)j * k, N);
            }
            y[k] = re;
            if (k > 0 && 2 * k != N) y[N - k] = im;
        }
        break;
    case R2R_HC2R:   /* x_j = r_0 + sum_k 2 (r_k cos - i_k sin) + r_{N/2} (-1)^j */
        for (int j = 0; j < N; ++j) {
            double s = x[0];
            for (int k = 1; 2 * k < N; ++k)
                s += 2.0 * (x[k] * cospi_frac(2 * (int64_t)j * k, N) - x[N - k] * sinpi_frac(2 * (int64_t)j * k, N));
            if (N % 2 == 0) s += (j % 2 ? -1.0 : 1.0) * x[N / 2];
            y[j] = s;
        }
        break;
    case R2R_RODFT00:   /* DST-I: 2 sum x_j sin(pi (j+1)(k+1)/(N+1)) */
        for (int k = 0; k < N; ++k) {
            double s = 0.0;
            for (int j = 0; j < N; ++j) s += x[j] * sinpi_frac((int64_t)(j + 1) * (k + 1), N + 1);
            y[k] = 2.0 * s;
        }
        break;
    case R2R_REDFT00:   /* DCT-I: x_0 + (-1)^k x_{N-1} + 2 sum_{j=1}^{N-2} x_j cos(pi jk/(N-1)) */
        for (int k = 0; k < N; ++k) {
            double s = 0.0;
            for (int j = 1; j < N - 1; ++j) s += x[j] * cospi_frac((int64_t)j * k, N - 1);
            y[k] = x[0] + (k % 2 ? -1.0 : 1.0) * x[N - 1] + 2.0 * s;
        }
        break;
    case R2R_RODFT01:   /* DST-III: (-1)^k x_{N-1} + 2 sum_{j=0}^{N-2} x_j sin(pi (j+1)(2k+1)/(2N)) */
        for (int k = 0; k < N; ++k) {
            double s = 0.0;
            for (int j = 0; j < N - 1; ++j) s += x[j] * sinpi_frac((int64_t)(j + 1) * (2 * k + 1), 2 * N);
            y[k] = (k % 2 ? -1.0 : 1.0) * x[N - 1] + 2.0 * s;
        }
        break;
    case R2R_RODFT10:   /* DST-II: 2 sum x_j sin(pi (2j+1)(k+1)/(2N)) */
        for (int k = 0; k < N; ++k) {
            double s = 0.0;
            for (int j = 0; j < N; ++j) s += x[j] * sinpi_frac((int64_t)(2 * j + 1) * (k + 1), 2 * N);
            y[k] = 2.0 * s;
        }
        break;
    case R2R_REDFT01:   /* DCT-III: x_0 + 2 sum_{j=1}^{N-1} x_j cos(pi j(2k+1)/(2N)) */
        for (int k = 0; k < N; ++k) {
            double s = 0.0;
            for (int j = 1; j < N; ++j) s += x[j] * cospi_frac((int64_t)j * (2 * k + 1), 2 * N);
            y[k] = x[0] + 2.0 * s;
        }
        break;
    case R2R_REDFT10:   /* DCT-II: 2 sum x_j cos(pi (2j+1)k/(2N)) */
        for (int k = 0; k < N; ++k) {
            double s = 0.0;
            for (int j = 0; j < N; ++j) s += x[j] * cospi_frac((int64_t)(2 * j + 1) * k, 2 * N);
            y[k] = 2.0 * s;
        }
        break;
    default:
        break;
    }
}

/* convert_fft_type (mpi_fftw3_solver.f90:151-207) for the global block 0..n. */
typedef struct {
    int fwd, bwd, ls, L;
    double norm;
} bc_axis;

static int bc_axis_of(int kind, int n, bc_axis *a)
{
    switch (kind) {
    case ORC_BC_PERIODIC: a->fwd = R2R_R2HC; a->bwd = R2R_HC2R; a->ls = 0; a->L = n; a->norm = (double)a->L; break;
    case ORC_BC_DIRICHLET: a->fwd = a->bwd = R2R_RODFT00; a->ls = 1; a->L = n - 1; a->norm = 2.0 * (a->L + 1.0); break;
    case ORC_BC_NEUMANN: a->fwd = a->bwd = R2R_REDFT00; a->ls = 0; a->L = n + 1; a->norm = 2.0 * (a->L - 1.0); break;
    case ORC_BC_DIRICHLET_NEUMANN: a->fwd = R2R_RODFT01; a->bwd = R2R_RODFT10; a->ls = 1; a->L = n; a->norm = 2.0 * a->L; break;
    case ORC_BC_NEUMANN_DIRICHLET: a->fwd = R2R_REDFT01; a->bwd = R2R_REDFT10; a->ls = 0; a->L = n; a->norm = 2.0 * a->L; break;
    default: return -1;
    }
    return a->L >= 1 && !(kind == ORC_BC_NEUMANN && a->L < 2) ? 0 : -1;
}

/* calc_wave_number (poisson_solver3d.f90:104-132) with the reference's pi. */
static double bc_wave_number(int k, int n, int kind)
{
    switch (kind) {
    case ORC_BC_PERIODIC:
        if (k <= n / 2) return 2.0 * sin(REF_PI * k / (double)n);
        return 2.0 * sin(REF_PI * (n - k) / (double)n);
    case ORC_BC_DIRICHLET: return 2.0 * (cos(REF_PI * (k + 1) / (double)(n + 1)) - 1.0);
    case ORC_BC_NEUMANN: return 2.0 * (cos(REF_PI * k / (double)n) - 1.0);
    case ORC_BC_DIRICHLET_NEUMANN:
    case ORC_BC_NEUMANN_DIRICHLET: return 2.0 * (cos(REF_PI * (k + 0.5) / (double)(n + 1)) - 1.0);
    }
    return 0.0;
}

/* The Laplacian's eigenvalue (negated) of logical mode i of each kind. */
static double bc_eigenvalue(int i, int n, int kind)
{
    switch (kind) {
    case ORC_BC_PERIODIC: {
        const double w = bc_wave_number(i, n, kind);
        return w * w;
    }
    case ORC_BC_DIRICHLET: return 2.0 - 2.0 * cos(REF_PI * (i + 1) / (double)n);
    case ORC_BC_NEUMANN: return 2.0 - 2.0 * cos(REF_PI * i / (double)n);
    case ORC_BC_DIRICHLET_NEUMANN:
    case ORC_BC_NEUMANN_DIRICHLET: return 2.0 - 2.0 * cos(REF_PI * (i + 0.5) / (double)n);
    }
    return 0.0;
}

/* calc_boundary_term (poisson_solver3d.f90:81-102). */
static void bc_terms(int kind, const double bv[2], double t[2])
{
    switch (kind) {
    case ORC_BC_PERIODIC: t[0] = bv[0]; t[1] = bv[1]; break;
    case ORC_BC_DIRICHLET: t[0] = -bv[0]; t[1] = -bv[1]; break;
    case ORC_BC_NEUMANN: t[0] = 2.0 * bv[0]; t[1] = -2.0 * bv[1]; break;
    default: t[0] = -bv[0]; t[1] = -2.0 * bv[1]; break;   /* both mixed kinds */
    }
}

static int bc_has_wall_lo(int kind) { return kind == ORC_BC_DIRICHLET || kind == ORC_BC_DIRICHLET_NEUMANN; }
static int bc_has_wall_hi(int kind) { return kind == ORC_BC_DIRICHLET || kind == ORC_BC_NEUMANN_DIRICHLET; }

/* Applies one 1-D transform along `axis` of a (L0, L1, L2) array, x fastest. */
static void bc_transform_axis(double *a, const int L[3], int axis, int kind)
{
    const int64_t s[3] = {1, L[0], (int64_t)L[0] * L[1]};
    const int o1 = axis == 0 ? 1 : 0, o2 = axis == 2 ? 1 : 2;
    const int N = L[axis];
    double *x = (double *)malloc(sizeof(double) * N), *y = (double *)malloc(sizeof(double) * N);
    for (int q = 0; q < L[o2]; ++q)
        for (int p = 0; p < L[o1]; ++p) {
            const int64_t base = p * s[o1] + q * s[o2];
            for (int j = 0; j < N; ++j) x[j] = a[base + j * s[axis]];
            orc_r2r_1d(kind, x, y, N);
            for (int j = 0; j < N; ++j) a[base + j * s[axis]] = y[j];
        }
    free(x);
    free(y);
}

int orc_poisson_bc(const int n[3], const int kinds[3], const double bv[6], int corrected, const double *rho,
                   double *phi, double *e)
{
    bc_axis ax[3];
    for (int d = 0; d < 3; ++d)
        if (n[d] < 1 || bc_axis_of(kinds[d], n[d], &ax[d]) != 0) return -1;
    const int B[3] = {n[0] + 1, n[1] + 1, n[2] + 1};
    const int64_t nb = (int64_t)B[0] * B[1] * B[2];
    double *w = (double *)malloc(sizeof(double) * nb);
    memcpy(w, rho, sizeof(double) * nb);   /* phi = rho (poisson_solver3d.f90:147) */
#define BIDX(i, j, k) ((i) + (int64_t)B[0] * ((j) + (int64_t)B[1] * (k)))
    for (int d = 0; d < 3; ++d) {
        double t[2];
        int lo = 0, hi = n[d];
        bc_terms(kinds[d], bv + 2 * d, t);
        if (corrected) {
            /* A Dirichlet wall value is the wall's potential: it enters the
             * equation of the adjacent interior node.  A Neumann value keeps the
             * reference's meaning (2 bv at the low wall, -2 bv at the high one). */
            if (kinds[d] == ORC_BC_PERIODIC) continue;
            if (bc_has_wall_lo(kinds[d])) { t[0] = bv[2 * d]; lo = 1; }
            else t[0] = 2.0 * bv[2 * d];
            if (bc_has_wall_hi(kinds[d])) { t[1] = bv[2 * d + 1]; hi = n[d] - 1; }
            else t[1] = -2.0 * bv[2 * d + 1];
        }
        /* the face planes of the block (poisson_solver3d.f90:156-168) */
        for (int k = 0; k < B[2]; ++k)
            for (int j = 0; j < B[1]; ++j)
                for (int i = 0; i < B[0]; ++i) {
                    const int g = d == 0 ? i : d == 1 ? j : k;
                    if (g == lo) w[BIDX(i, j, k)] += t[0];
                    if (g == hi) w[BIDX(i, j, k)] += t[1];
                }
    }
    const int L[3] = {ax[0].L, ax[1].L, ax[2].L};
    const int64_t nl = (int64_t)L[0] * L[1] * L[2];
    double *a = (double *)malloc(sizeof(double) * nl);
    for (int k = 0; k < L[2]; ++k)
        for (int j = 0; j < L[1]; ++j)
            for (int i = 0; i < L[0]; ++i)
                a[i + (int64_t)L[0] * (j + (int64_t)L[1] * k)] = w[BIDX(i + ax[0].ls, j + ax[1].ls, k + ax[2].ls)];
    for (int d = 0; d < 3; ++d) bc_transform_axis(a, L, d, ax[d].fwd);
    for (int k = 0; k < L[2]; ++k)
        for (int j = 0; j < L[1]; ++j)
            for (int i = 0; i < L[0]; ++i) {
                const int64_t at = i + (int64_t)L[0] * (j + (int64_t)L[1] * k);
                double den;
                if (corrected) {
                    den = bc_eigenvalue(i, n[0], kinds[0]) + bc_eigenvalue(j, n[1], kinds[1]) +
                          bc_eigenvalue(k, n[2], kinds[2]);
                    a[at] = den == 0.0 ? 0.0 : a[at] / den;
                } else {
                    /* modified_wave_number at the element's global index (:62-78) */
                    const double wx = bc_wave_number(i + ax[0].ls, n[0], kinds[0]);
                    const double wy = bc_wave_number(j + ax[1].ls, n[1], kinds[1]);
                    const double wz = bc_wave_number(k + ax[2].ls, n[2], kinds[2]);
                    den = wx * wx + wy * wy + wz * wz;
                    a[at] = a[at] / den;
                }
            }
    /* element (0,0,0) of the block (:194-198): inside the transform only when
     * every logical range starts at node 0 */
    if (!corrected && ax[0].ls == 0 && ax[1].ls == 0 && ax[2].ls == 0) a[0] = 0.0;
    for (int d = 2; d >= 0; --d) bc_transform_axis(a, L, d, ax[d].bwd);
    const double norm = ax[0].norm * ax[1].norm * ax[2].norm;
    for (int k = 0; k < B[2]; ++k)
        for (int j = 0; j < B[1]; ++j)
            for (int i = 0; i < B[0]; ++i) {
                int g[3] = {i, j, k};
                double wall = 0.0;
                int at_wall = 0;
                for (int d = 0; d < 3 && !at_wall; ++d) {
                    if (kinds[d] == ORC_BC_PERIODIC && g[d] == n[d]) g[d] = 0;
                    else if (bc_has_wall_lo(kinds[d]) && g[d] == 0) { at_wall = 1; wall = corrected ? bv[2 * d] : 0.0; }
                    else if (bc_has_wall_hi(kinds[d]) && g[d] == n[d]) { at_wall = 1; wall = corrected ? bv[2 * d + 1] : 0.0; }
                }
                double v = wall;
                if (!at_wall) {
                    const int64_t at = (g[0] - ax[0].ls) + (int64_t)L[0] * ((g[1] - ax[1].ls) + (int64_t)L[1] * (g[2] - ax[2].ls));
                    v = a[at] / norm;
                }
                phi[BIDX(i, j, k)] = v;
            }
    if (e) {
        for (int k = 0; k < B[2]; ++k)
            for (int j = 0; j < B[1]; ++j)
                for (int i = 0; i < B[0]; ++i) {
                    const int g[3] = {i, j, k};
                    for (int d = 0; d < 3; ++d) {
                        int gm[3] = {i, j, k}, gp[3] = {i, j, k};
                        double v;
                        const double p0 = phi[BIDX(i, j, k)];
                        if (kinds[d] == ORC_BC_PERIODIC) {
                            const int c = g[d] == n[d] ? 0 : g[d];
                            gm[d] = (c + n[d] - 1) % n[d];
                            gp[d] = (c + 1) % n[d];
                            v = 0.5 * ((phi[BIDX(gm[0], gm[1], gm[2])] - p0) + (p0 - phi[BIDX(gp[0], gp[1], gp[2])]));
                        } else if (g[d] == 0) {
                            gp[d] = 1;
                            v = p0 - phi[BIDX(gp[0], gp[1], gp[2])];
                        } else if (g[d] == n[d]) {
                            gm[d] = n[d] - 1;
                            v = phi[BIDX(gm[0], gm[1], gm[2])] - p0;
                        } else {
                            gm[d] = g[d] - 1;
                            gp[d] = g[d] + 1;
                            v = 0.5 * ((phi[BIDX(gm[0], gm[1], gm[2])] - p0) + (p0 - phi[BIDX(gp[0], gp[1], gp[2])]));
                        }
                        e[(int64_t)d * nb + BIDX(i, j, k)] = v;
                    }
                }
    }
#undef BIDX
    free(a);
    free(w);
    return 0;
}
