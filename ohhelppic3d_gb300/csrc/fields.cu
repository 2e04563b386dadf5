// fields.cu -- spectral Poisson solve and the E stencil.
//
// Reference: t_PoissonFieldSolver%solve (src/field_solver/poisson_field_solver.f90:90-175)
//   phi = rho; forward R2HC x3; divide by the modified wave number
//   sum_d (2 sin(pi k_d / n_d))^2 (poisson_solver3d.f90:104-117, :184-192); zero k = 0
//   (:194-198); backward HC2R x3 and divide by nx*ny*nz (mpi_fftw3_solver.f90:223-236);
//   then E_d[i] = phi[i] - phi[i+e_d] (:131-145) and E_d[i] = (E_d[i-e_d] + E_d[i]) / 2
//   (:157-171), which combine to E_d[i] = 0.5*((phi[i-e] - phi[i]) + (phi[i] - phi[i+e])).
//
// The tensor-product real half-complex basis of the reference and the R2C
// transform used here diagonalise the same periodic 7-point Laplacian, with the
// same eigenvalue per wave vector, so dividing the cuFFT half spectrum by that
// eigenvalue gives the reference's phi up to rounding.  The Green table holds
// 1/(eigenvalue * nx*ny*nz) in FP64 (0 at k = 0) and is built once on the device
// with the reference's truncated pi literal (src/utils/science_constants.f90:4).
#include <cuda_runtime.h>
#include <cufft.h>
#include <stdint.h>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

constexpr double kRefPi = 3.14159265358979;

__device__ __forceinline__ double wave_number(int k, int n)
{
    // poisson_solver3d.f90:114-117
    if (k <= n / 2) return 2.0 * sin(kRefPi * k / (double)n);
    return 2.0 * sin(kRefPi * (n - k) / (double)n);
}

__global__ void k_green(Geom g, double *green)
{
    const int64_t total = g.nspec;
    const double norm = (double)g.nx * (double)g.ny * (double)g.nz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int kx = (int)(i % g.nxh);
        const int ky = (int)((i / g.nxh) % g.ny);
        const int kz = (int)(i / ((int64_t)g.nxh * g.ny));
        if (kx == 0 && ky == 0 && kz == 0) {
            green[i] = 0.0;
            continue;
        }
        const double wx = wave_number(kx, g.nx), wy = wave_number(ky, g.ny), wz = wave_number(kz, g.nz);
        const double wn = wx * wx + wy * wy + wz * wz;
        green[i] = 1.0 / (wn * norm);
    }
}

__global__ void k_scale_z(cufftDoubleComplex *spec, const double *green, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double gf = green[i];
        cufftDoubleComplex v = spec[i];
        v.x *= gf;
        v.y *= gf;
        spec[i] = v;
    }
}

// FP32 spectrum scaled by the FP64 table in FP64 arithmetic.
__global__ void k_scale_c(cufftComplex *spec, const double *green, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double gf = green[i];
        cufftComplex v = spec[i];
        v.x = (float)((double)v.x * gf);
        v.y = (float)((double)v.y * gf);
        spec[i] = v;
    }
}

__device__ __forceinline__ int wrapn(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

// Padded E node t from phi (n^3), periodic ghosts included.
template <typename T, typename NodeT>
__device__ __forceinline__ void stencil_node(const Geom &g, const T *phi, NodeT *epad, int64_t t)
{
    const int64_t nxy = (int64_t)g.nx * g.ny;
    {
        const int px = (int)(t % g.gx);
        const int py = (int)((t / g.gx) % g.gy);
        const int pz = (int)(t / ((int64_t)g.gx * g.gy));
        const int i = wrapn(px - g.halo, g.nx), j = wrapn(py - g.halo, g.ny), k = wrapn(pz - g.halo, g.nz);
        const int im = i == 0 ? g.nx - 1 : i - 1, ip = i + 1 == g.nx ? 0 : i + 1;
        const int jm = j == 0 ? g.ny - 1 : j - 1, jp = j + 1 == g.ny ? 0 : j + 1;
        const int km = k == 0 ? g.nz - 1 : k - 1, kp = k + 1 == g.nz ? 0 : k + 1;
        const int64_t row = (int64_t)j * g.nx + (int64_t)k * nxy;
        const T p0 = phi[i + row];
        NodeT e;
        e.x = T(0.5) * ((phi[im + row] - p0) + (p0 - phi[ip + row]));
        e.y = T(0.5) * ((phi[i + (int64_t)jm * g.nx + (int64_t)k * nxy] - p0) +
                        (p0 - phi[i + (int64_t)jp * g.nx + (int64_t)k * nxy]));
        e.z = T(0.5) * ((phi[i + row - (int64_t)k * nxy + (int64_t)km * nxy] - p0) +
                        (p0 - phi[i + row - (int64_t)k * nxy + (int64_t)kp * nxy]));
        e.w = T(0);
        epad[t] = e;
    }
}

template <typename T, typename NodeT>
__global__ void k_stencil(Geom g, const T *phi, NodeT *epad)
{
    const int64_t total = (int64_t)g.gx * g.gy * g.gz;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
        stencil_node<T, NodeT>(g, phi, epad, t);
}

// ---- FP32 form: rho from the fixed-point weight sums ----
//
// rho = sum_s q_s * W_s * 2^-24 (W_s the species' integer weight sum at the
// node), rounded once to FP32.  Each charge is an integer mantissa times a power
// of two (from its bit pattern), so the sum is formed exactly in 128-bit integer
// arithmetic and rounded to nearest, ties to even: no FP64 arithmetic per node.
// Bounds: |m_s| < 2^53, W_s < 2^58 (every count is far below 2^34), the exponent
// spread at most kRhoMaxShift, at most 8 species: the sum stays below 2^126.
// Charges further apart in exponent (or subnormal), and sums outside the normal
// FP32 range, take the FP64 expression instead.
constexpr int kRhoMaxShift = 12;

struct RhoScale {
    long long m[OHPIC_MAX_SPECIES];
    int shift[OHPIC_MAX_SPECIES];
    int K;
    bool ok;
};

__device__ __forceinline__ RhoScale rho_scale(const double *q, int nsp)
{
    RhoScale r;
    r.ok = true;
    r.K = 0x7fffffff;
    int k[OHPIC_MAX_SPECIES];
    for (int s = 0; s < nsp; ++s) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(q[s]);
        const int e = (int)((b >> 52) & 0x7ffu);
        const long long mant = (long long)(b & ((1ull << 52) - 1));
        r.m[s] = 0;
        k[s] = 0;
        if (e == 0) {
            if (mant != 0) r.ok = false;   // subnormal charge
            continue;
        }
        if (e == 0x7ff) {
            r.ok = false;
            continue;
        }
        const long long m = mant | (1ll << 52);
        r.m[s] = (b >> 63) ? -m : m;
        k[s] = e - 1075 - 24;              // q_s * 2^-24 = m * 2^k
        r.K = min(r.K, k[s]);
    }
    for (int s = 0; s < nsp; ++s) {
        r.shift[s] = r.m[s] != 0 ? k[s] - r.K : 0;
        if (r.shift[s] > kRhoMaxShift) r.ok = false;
    }
    if (r.K == 0x7fffffff) r.K = 0;        // every charge zero: the sum is 0
    return r;
}

// acc * 2^K rounded to FP32, nearest with ties to even; false outside the
// normal range.
__device__ __forceinline__ bool i128_to_float_rne(__int128 acc, int K, float &out)
{
    if (acc == 0) {
        out = 0.f;
        return true;
    }
    const bool neg = acc < 0;
    const unsigned __int128 a = neg ? (unsigned __int128)(-acc) : (unsigned __int128)acc;
    const unsigned long long hi = (unsigned long long)(a >> 64), lo = (unsigned long long)a;
    int msb = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    unsigned int mant;
    if (msb <= 23) {
        mant = (unsigned int)(lo << (23 - msb));
    } else {
        const int sh = msb - 23;
        const unsigned __int128 one = 1;
        const unsigned __int128 rem = a & ((one << sh) - 1);
        const unsigned __int128 half = one << (sh - 1);
        mant = (unsigned int)(a >> sh);
        if (rem > half || (rem == half && (mant & 1u))) {
            ++mant;
            if (mant == (1u << 24)) {
                mant >>= 1;
                ++msb;
            }
        }
    }
    const int be = msb + K + 127;
    if (be < 1 || be > 254) return false;
    out = __uint_as_float((neg ? 0x80000000u : 0u) | ((unsigned)be << 23) | (mant & 0x7fffffu));
    return true;
}

// rho at one node: w[s * stride] is species s's weight sum.
__device__ __forceinline__ float node_rho(const unsigned long long *w, int64_t stride, int nsp, const double *q,
                                          const RhoScale &r)
{
    if (r.ok) {
        __int128 acc = 0;
        for (int s = 0; s < nsp; ++s) {
            const long long m = r.m[s];
            if (m == 0) continue;
            // |m| * W as one 64 x 64 -> 128-bit product, then the species' shift
            const unsigned long long W = w[s * stride];
            const unsigned long long am = (unsigned long long)(m < 0 ? -m : m);
            unsigned __int128 p = ((unsigned __int128)__umul64hi(am, W) << 64) | (unsigned __int128)(am * W);
            p <<= r.shift[s];
            acc = m < 0 ? acc - (__int128)p : acc + (__int128)p;
        }
        float v;
        if (i128_to_float_rne(acc, r.K, v)) return v;
    }
    double acc = 0.0;
    for (int s = 0; s < nsp; ++s) acc += q[s] * (double)w[s * stride];
    return (float)(acc * kWeightUnit);
}

// node_rho of one or two species whose weight sums are already in registers.
__device__ __forceinline__ float node_rho2(const unsigned long long W[2], int nsp, const double *q, const RhoScale &r)
{
    if (r.ok) {
        __int128 acc = 0;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const long long m = s < nsp ? r.m[s] : 0;
            if (m == 0) continue;
            const unsigned long long am = (unsigned long long)(m < 0 ? -m : m);
            unsigned __int128 p = ((unsigned __int128)__umul64hi(am, W[s]) << 64) | (unsigned __int128)(am * W[s]);
            p <<= r.shift[s];
            acc = m < 0 ? acc - (__int128)p : acc + (__int128)p;
        }
        float v;
        if (i128_to_float_rne(acc, r.K, v)) return v;
    }
    double acc = 0.0;
#pragma unroll
    for (int s = 0; s < 2; ++s)
        if (s < nsp) acc += q[s] * (double)W[s];
    return (float)(acc * kWeightUnit);
}

// ---- pooled fields: many runs of one grid size, slot = blockIdx.y; on[slot] == 0 skips ----

// rho of every active slot from its fixed-point weight sums (nsp species per slot,
// charges q[slot * nsp + s]); the sums are cleared for the next deposit.
__global__ void k_pool_rho(unsigned long long *w, int64_t ncell, int nsp, const double *q, const int *on,
                           float *rho)
{
    const int slot = blockIdx.y;
    if (on && !on[slot]) return;
    w += (int64_t)slot * nsp * ncell;
    rho += (int64_t)slot * ncell;
    q += (int64_t)slot * nsp;
    __shared__ RhoScale r;
    if (threadIdx.x == 0) r = rho_scale(q, nsp);
    __syncthreads();
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ncell; t += (int64_t)gridDim.x * blockDim.x) {
        rho[t] = node_rho(w + t, ncell, nsp, q, r);
        for (int s = 0; s < nsp; ++s) w[s * ncell + t] = 0ull;
    }
}

__global__ void k_pool_scale(cufftComplex *spec, int64_t nspec, const double *green, const int *on)
{
    const int slot = blockIdx.y;
    if (on && !on[slot]) return;
    spec += (int64_t)slot * nspec;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nspec; i += (int64_t)gridDim.x * blockDim.x) {
        const double gf = green[i];
        cufftComplex v = spec[i];
        v.x = (float)((double)v.x * gf);
        v.y = (float)((double)v.y * gf);
        spec[i] = v;
    }
}

__global__ void k_pool_stencil(Geom g, const float *phi, float4 *epad, const int *on)
{
    const int slot = blockIdx.y;
    if (on && !on[slot]) return;
    const int64_t total = (int64_t)g.gx * g.gy * g.gz;
    phi += (int64_t)slot * g.ncell;
    epad += (int64_t)slot * total;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
        stencil_node<float, float4>(g, phi, epad, t);
}

// One n^3 FP64 component array -> that component of every padded E node (uploaded E).
template <typename T, typename NodeT>
__global__ void k_fill_epad(Geom g, const double *src, int comp, NodeT *epad)
{
    const int64_t total = (int64_t)g.gx * g.gy * g.gz;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int px = (int)(t % g.gx);
        const int py = (int)((t / g.gx) % g.gy);
        const int pz = (int)(t / ((int64_t)g.gx * g.gy));
        const int i = wrapn(px - g.halo, g.nx), j = wrapn(py - g.halo, g.ny), k = wrapn(pz - g.halo, g.nz);
        const T v = (T)src[i + (int64_t)g.nx * (j + (int64_t)g.ny * k)];
        if (comp == 0) epad[t].x = v;
        else if (comp == 1) epad[t].y = v;
        else epad[t].z = v;
    }
}

// Interior of the padded E -> one FP64 component array.
template <typename NodeT>
__global__ void k_epad_component(Geom g, const NodeT *epad, int comp, double *out)
{
    const int64_t total = g.ncell;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.nx);
        const int j = (int)((t / g.nx) % g.ny);
        const int k = (int)(t / ((int64_t)g.nx * g.ny));
        const NodeT e = epad[(i + g.halo) + (int64_t)g.gx * ((j + g.halo) + (int64_t)g.gy * (k + g.halo))];
        out[t] = comp == 0 ? (double)e.x : comp == 1 ? (double)e.y : (double)e.z;
    }
}

template <typename T>
__global__ void k_to_double(const T *in, double *out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}

template <typename T>
__global__ void k_from_double(const double *in, T *out, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (T)in[i];
}

// FP64 reductions: sum of rho and 0.5 * sum |E|^2 over interior nodes.
template <typename T, typename NodeT>
__global__ void k_field_sums(Geom g, const T *rho, const NodeT *epad, double *charge, double *energy)
{
    double q = 0.0, e2 = 0.0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < g.ncell; t += (int64_t)gridDim.x * blockDim.x) {
        q += (double)rho[t];
        const int i = (int)(t % g.nx);
        const int j = (int)((t / g.nx) % g.ny);
        const int k = (int)(t / ((int64_t)g.nx * g.ny));
        const NodeT e = epad[(i + g.halo) + (int64_t)g.gx * ((j + g.halo) + (int64_t)g.gy * (k + g.halo))];
        e2 += (double)e.x * (double)e.x + (double)e.y * (double)e.y + (double)e.z * (double)e.z;
    }
    for (int o = 16; o > 0; o >>= 1) {
        q += __shfl_xor_sync(0xffffffffu, q, o);
        e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(charge, q);
        atomicAdd(energy, 0.5 * e2);
    }
}

// FP32 form: rho = sum_s q_s * W_s * 2^-24 from the fixed-point weight sums,
// summed exactly and rounded once to FP32 (node_rho).
struct SpeciesCharges {
    double q[OHPIC_MAX_SPECIES];
    int nspecies;
};

// Four nodes per thread per iteration, every weight-sum load of the four issued
// before the first node is formed: one node at a time, the kernel waited on two
// dependent-free loads per node and ran at a third of its bytes' bandwidth.
__global__ void k_wsum_to_rho(const unsigned long long *w, int64_t ncell, SpeciesCharges sc, float *rho)
{
    constexpr int U = 4;
    __shared__ RhoScale r;
    if (threadIdx.x == 0) r = rho_scale(sc.q, sc.nspecies);
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ncell; t += U * stride) {
        unsigned long long W[U][2];
        bool in[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t i = t + u * stride;
            in[u] = i < ncell;
            W[u][0] = in[u] ? w[i] : 0ull;
            W[u][1] = in[u] && sc.nspecies > 1 ? w[ncell + i] : 0ull;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (!in[u]) continue;
            const int64_t i = t + u * stride;
            rho[i] = sc.nspecies <= 2 ? node_rho2(W[u], sc.nspecies, sc.q, r) : node_rho(w + i, ncell, sc.nspecies, sc.q, r);
        }
    }
}

// FP64 form: rho = (sum_s q_s W_s) 2^-48 from the species' 2^-48 fixed-point
// weight sums, the species added in a fixed order, so rho is bit-reproducible.
__global__ void k_wsum_to_rho64(const unsigned long long *w, int64_t ncell, SpeciesCharges sc, double *rho)
{
    constexpr double kUnit48 = 1.0 / 281474976710656.0;   // 2^-48
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ncell; t += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int s = 0; s < sc.nspecies; ++s) acc += sc.q[s] * (double)w[s * ncell + t];
        rho[t] = acc * kUnit48;
    }
}

int blocks_for(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return b < 1 ? 1 : (int)b;
}

}  // namespace

// Materialise rho from the fixed-point weight sums left by the last deposit.
void ensure_rho(ohpic_ctx *c)
{
    if (!c->rho_from_wsum) return;
    SpeciesCharges sc;
    sc.nspecies = c->cfg.nspecies;
    for (int s = 0; s < OHPIC_MAX_SPECIES; ++s) sc.q[s] = s < sc.nspecies ? c->cfg.q[s] : 0.0;
    if (c->cfg.precision == OHPIC_FP32)
        k_wsum_to_rho<<<blocks_for(c->g.ncell), 256, 0, c->stream>>>(c->wsum, c->g.ncell, sc, (float *)c->rho);
    else
        k_wsum_to_rho64<<<blocks_for(c->g.ncell), 256, 0, c->stream>>>(c->wsum, c->g.ncell, sc, (double *)c->rho);
    ++c->launches;
    c->rho_from_wsum = false;
}

int fields_setup(ohpic_ctx *c)
{
    const Geom &g = c->g;
    cufftResult r;
    if (c->cfg.precision == OHPIC_FP64) {
        r = cufftPlan3d(&c->plan_r2c, g.nz, g.ny, g.nx, CUFFT_D2Z);
        if (r == CUFFT_SUCCESS) r = cufftPlan3d(&c->plan_c2r, g.nz, g.ny, g.nx, CUFFT_Z2D);
    } else {
        r = cufftPlan3d(&c->plan_r2c, g.nz, g.ny, g.nx, CUFFT_R2C);
        if (r == CUFFT_SUCCESS) r = cufftPlan3d(&c->plan_c2r, g.nz, g.ny, g.nx, CUFFT_C2R);
    }
    if (r != CUFFT_SUCCESS) {
        c->err = "cufftPlan3d failed (" + std::to_string((int)r) + ")";
        return OHPIC_ERR_CUDA;
    }
    c->plans_made = true;
    cufftSetStream(c->plan_r2c, c->stream);
    cufftSetStream(c->plan_c2r, c->stream);
    k_green<<<blocks_for(g.nspec), 256, 0, c->stream>>>(g, c->green);
    ++c->launches;
    return OHPIC_OK;
}

void fields_teardown(ohpic_ctx *c)
{
    if (c->plans_made) {
        cufftDestroy(c->plan_r2c);
        cufftDestroy(c->plan_c2r);
        c->plans_made = false;
    }
}

int solve_fields(ohpic_ctx *c)
{
    const Geom &g = c->g;
    ensure_rho(c);
    cufftResult r;
    if (c->cfg.precision == OHPIC_FP64) {
        r = cufftExecD2Z(c->plan_r2c, (cufftDoubleReal *)c->rho, (cufftDoubleComplex *)c->spec);
        if (r != CUFFT_SUCCESS) goto fail;
        k_scale_z<<<blocks_for(g.nspec), 256, 0, c->stream>>>((cufftDoubleComplex *)c->spec, c->green, g.nspec);
        r = cufftExecZ2D(c->plan_c2r, (cufftDoubleComplex *)c->spec, (cufftDoubleReal *)c->phi);
        if (r != CUFFT_SUCCESS) goto fail;
        k_stencil<double, dnode><<<blocks_for((int64_t)g.gx * g.gy * g.gz), 256, 0, c->stream>>>(
            g, (const double *)c->phi, (dnode *)c->epad);
    } else {
        r = cufftExecR2C(c->plan_r2c, (cufftReal *)c->rho, (cufftComplex *)c->spec);
        if (r != CUFFT_SUCCESS) goto fail;
        k_scale_c<<<blocks_for(g.nspec), 256, 0, c->stream>>>((cufftComplex *)c->spec, c->green, g.nspec);
        r = cufftExecC2R(c->plan_c2r, (cufftComplex *)c->spec, (cufftReal *)c->phi);
        if (r != CUFFT_SUCCESS) goto fail;
        k_stencil<float, float4><<<blocks_for((int64_t)g.gx * g.gy * g.gz), 256, 0, c->stream>>>(
            g, (const float *)c->phi, (float4 *)c->epad);
    }
    c->launches += 2;
    return OHPIC_OK;
fail:
    c->err = "cuFFT exec failed (" + std::to_string((int)r) + ")";
    return OHPIC_ERR_CUDA;
}

void launch_zero(ohpic_ctx *c, void *p, int64_t bytes) { cudaMemsetAsync(p, 0, (size_t)bytes, c->stream); }

// ---- pooled solve (serve.cu): returns the number of launches, or -1 on a cuFFT error ----

int pool_green(cudaStream_t st, const Geom &g, double *green)
{
    k_green<<<blocks_for(g.nspec), 256, 0, st>>>(g, green);
    return 1;
}

int pool_solve(cudaStream_t st, const FieldPool &p)
{
    const Geom &g = p.g;
    const unsigned slots = (unsigned)p.slots;
    auto grid = [&](int64_t n) {
        int64_t b = (n + 255) / 256;
        const int64_t cap = (152 * 16 + slots - 1) / slots;
        if (b > cap) b = cap;
        return dim3((unsigned)(b < 1 ? 1 : b), slots);
    };
    k_pool_rho<<<grid(g.ncell), 256, 0, st>>>(p.wsum, g.ncell, p.nsp, p.q, p.on, p.rho);
    if (cufftExecR2C(p.r2c, p.rho, p.spec) != CUFFT_SUCCESS) return -1;
    k_pool_scale<<<grid(g.nspec), 256, 0, st>>>(p.spec, g.nspec, p.green, p.on);
    if (cufftExecC2R(p.c2r, p.spec, p.phi) != CUFFT_SUCCESS) return -1;
    k_pool_stencil<<<grid((int64_t)g.gx * g.gy * g.gz), 256, 0, st>>>(g, p.phi, p.epad, p.on);
    return 5;
}

// rho of one slot from its weight sums (the deposit of the run's last step).
void pool_slot_rho(cudaStream_t st, const FieldPool &p, int slot)
{
    const Geom &g = p.g;
    k_pool_rho<<<dim3(blocks_for(g.ncell), 1), 256, 0, st>>>(p.wsum + (int64_t)slot * p.nsp * g.ncell, g.ncell,
                                                             p.nsp, p.q + (int64_t)slot * p.nsp, nullptr,
                                                             p.rho + (int64_t)slot * g.ncell);
}

// One slot's fields as FP64 arrays: rho, phi, Ex, Ey, Ez (5 * ncell doubles).
void pool_slot_fields(cudaStream_t st, const FieldPool &p, int slot, double *dst)
{
    const Geom &g = p.g;
    const int64_t n = g.ncell, npad = (int64_t)g.gx * g.gy * g.gz;
    k_to_double<float><<<blocks_for(n), 256, 0, st>>>(p.rho + slot * n, dst, n);
    k_to_double<float><<<blocks_for(n), 256, 0, st>>>(p.phi + slot * n, dst + n, n);
    for (int c = 0; c < 3; ++c)
        k_epad_component<float4><<<blocks_for(n), 256, 0, st>>>(g, p.epad + slot * npad, c, dst + (2 + c) * n);
}

// Charge and field energy of one slot (FP64 sums into d->charge, d->field_energy).
void pool_slot_sums(cudaStream_t st, const FieldPool &p, int slot, DevDiag *d)
{
    const Geom &g = p.g;
    cudaMemsetAsync(&d->charge, 0, 2 * sizeof(double), st);
    k_field_sums<float, float4><<<blocks_for(g.ncell), 256, 0, st>>>(
        g, p.rho + slot * g.ncell, p.epad + slot * ((int64_t)g.gx * g.gy * g.gz), &d->charge, &d->field_energy);
}

void launch_field_energy(ohpic_ctx *c)
{
    const Geom &g = c->g;
    ensure_rho(c);
    cudaMemsetAsync(&c->diag->charge, 0, 2 * sizeof(double), c->stream);
    if (c->cfg.precision == OHPIC_FP64)
        k_field_sums<double, dnode><<<blocks_for(g.ncell), 256, 0, c->stream>>>(
            g, (const double *)c->rho, (const dnode *)c->epad, &c->diag->charge, &c->diag->field_energy);
    else
        k_field_sums<float, float4><<<blocks_for(g.ncell), 256, 0, c->stream>>>(
            g, (const float *)c->rho, (const float4 *)c->epad, &c->diag->charge, &c->diag->field_energy);
    ++c->launches;
}

// Field transfers through a device staging buffer of >= 3*ncell doubles.
void field_to_double(ohpic_ctx *c, int which, double *dst)
{
    const Geom &g = c->g;
    const bool f64 = c->cfg.precision == OHPIC_FP64;
    if (which == OHPIC_RHO) ensure_rho(c);
    if (which == OHPIC_RHO || which == OHPIC_PHI) {
        const void *src = which == OHPIC_RHO ? c->rho : c->phi;
        if (f64)
            cudaMemcpyAsync(dst, src, sizeof(double) * g.ncell, cudaMemcpyDeviceToDevice, c->stream);
        else
            k_to_double<float><<<blocks_for(g.ncell), 256, 0, c->stream>>>((const float *)src, dst, g.ncell);
    } else {
        const int comp = which - OHPIC_EX;
        if (f64)
            k_epad_component<dnode><<<blocks_for(g.ncell), 256, 0, c->stream>>>(g, (const dnode *)c->epad, comp, dst);
        else
            k_epad_component<float4><<<blocks_for(g.ncell), 256, 0, c->stream>>>(g, (const float4 *)c->epad, comp,
                                                                                 dst);
    }
    ++c->launches;
}

void field_from_double(ohpic_ctx *c, int which, const double *src)
{
    const Geom &g = c->g;
    const bool f64 = c->cfg.precision == OHPIC_FP64;
    if (which == OHPIC_RHO || which == OHPIC_PHI) {
        void *dst = which == OHPIC_RHO ? c->rho : c->phi;
        if (f64)
            cudaMemcpyAsync(dst, src, sizeof(double) * g.ncell, cudaMemcpyDeviceToDevice, c->stream);
        else
            k_from_double<float><<<blocks_for(g.ncell), 256, 0, c->stream>>>(src, (float *)dst, g.ncell);
    } else {
        const int comp = which - OHPIC_EX;
        if (f64)
            k_fill_epad<double, dnode><<<blocks_for((int64_t)g.gx * g.gy * g.gz), 256, 0, c->stream>>>(
                g, src, comp, (dnode *)c->epad);
        else
            k_fill_epad<float, float4><<<blocks_for((int64_t)g.gx * g.gy * g.gz), 256, 0, c->stream>>>(
                g, src, comp, (float4 *)c->epad);
    }
    ++c->launches;
}

}  // namespace ohpic
