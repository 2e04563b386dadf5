// noalloc.cu -- a CIC charge deposit that allocates no device memory.
//
// Some callers cannot let a library allocate GPU memory: codes that size all
// device memory once at start-up through their own pool and treat any later
// cudaMalloc as an error, or that run the deposit inside a step where an
// allocation could fail or synchronise the device.  ohpic_scatter_noalloc
// serves them.  The caller passes the particle positions and the rho array (both
// device memory it owns).  The one scratch buffer, the per-node 64-bit
// fixed-point weight sums, is the file-scope array below.  Every GPU that loads
// the library holds it (16 MiB) until the process exits.
//
// Algorithm: a fixed-point CIC deposit like the FP32 form's shared box
// (push_f32.cu).  Each particle's 8 weights are rounded to units of 2^-24, the
// largest corner takes the rounding remainder so they sum to exactly 2^24, and
// they are added with 64-bit integer atomics.  A second kernel adds
// charge * sum * 2^-24 to rho and clears the scratch for the next call, so the
// result does not depend on the order of the atomics.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

constexpr int64_t kNoAllocMaxNodes = (int64_t)1 << 21;   // e.g. 128^3 nodes

// Scratch shared by every call on a device; zero at load and cleared by each call.
static __device__ __align__(256) unsigned long long g_noalloc_sum[kNoAllocMaxNodes];

__device__ __forceinline__ double wrap_pos(double p, int n)
{
    if (p >= 0.0 && p < (double)n) return p;
    double w = fmod(p, (double)n);
    if (w < 0.0) w += (double)n;
    return w >= (double)n ? 0.0 : w;
}

__global__ void k_noalloc_deposit(const double *x, const double *y, const double *z, int64_t n, int nx, int ny,
                                  int nz, int weights, unsigned long long *sum)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double px = x[i], py = y[i], pz = z[i];
        if (!(isfinite(px) && isfinite(py) && isfinite(pz))) continue;   // nothing to deposit
        const double fx = wrap_pos(px, nx), fy = wrap_pos(py, ny), fz = wrap_pos(pz, nz);
        int ix = (int)fx, iy = (int)fy, iz = (int)fz;
        ix = ix >= nx ? nx - 1 : ix;
        iy = iy >= ny ? ny - 1 : iy;
        iz = iz >= nz ? nz - 1 : iz;
        const double rx = fx - ix, ry = fy - iy, rz = fz - iz;
        // node floor(x) gets r under the reference convention, 1-r under the standard one
        const double wx0 = weights == OHPIC_WEIGHTS_REFERENCE ? rx : 1.0 - rx, wx1 = 1.0 - wx0;
        const double wy0 = weights == OHPIC_WEIGHTS_REFERENCE ? ry : 1.0 - ry, wy1 = 1.0 - wy0;
        const double wz0 = weights == OHPIC_WEIGHTS_REFERENCE ? rz : 1.0 - rz, wz1 = 1.0 - wz0;
        const double f[8] = {wx0 * wy0 * wz0, wx1 * wy0 * wz0, wx0 * wy1 * wz0, wx1 * wy1 * wz0,
                             wx0 * wy0 * wz1, wx1 * wy0 * wz1, wx0 * wy1 * wz1, wx1 * wy1 * wz1};
        unsigned u[8], total = 0;
#pragma unroll
        for (int v = 0; v < 8; ++v) {
            u[v] = (unsigned)__double2uint_rn(f[v] * (double)kWeightScale);
            total += u[v];
        }
        const int big = (wx1 > wx0 ? 1 : 0) + (wy1 > wy0 ? 2 : 0) + (wz1 > wz0 ? 4 : 0);
        const unsigned fix = (1u << 24) - total;
#pragma unroll
        for (int v = 0; v < 8; ++v) u[v] += v == big ? fix : 0u;
        const int ix1 = ix + 1 == nx ? 0 : ix + 1, iy1 = iy + 1 == ny ? 0 : iy + 1, iz1 = iz + 1 == nz ? 0 : iz + 1;
        const int64_t y0 = (int64_t)iy * nx, y1 = (int64_t)iy1 * nx;
        const int64_t z0 = (int64_t)iz * nx * ny, z1 = (int64_t)iz1 * nx * ny;
        atomicAdd(sum + ix + y0 + z0, (unsigned long long)u[0]);
        atomicAdd(sum + ix1 + y0 + z0, (unsigned long long)u[1]);
        atomicAdd(sum + ix + y1 + z0, (unsigned long long)u[2]);
        atomicAdd(sum + ix1 + y1 + z0, (unsigned long long)u[3]);
        atomicAdd(sum + ix + y0 + z1, (unsigned long long)u[4]);
        atomicAdd(sum + ix1 + y0 + z1, (unsigned long long)u[5]);
        atomicAdd(sum + ix + y1 + z1, (unsigned long long)u[6]);
        atomicAdd(sum + ix1 + y1 + z1, (unsigned long long)u[7]);
    }
}

// rho += charge * sum * 2^-24, and the scratch goes back to zero for the next call.
__global__ void k_noalloc_finish(unsigned long long *sum, int64_t ncell, double charge, double *rho)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ncell; t += (int64_t)gridDim.x * blockDim.x) {
        const unsigned long long s = sum[t];
        if (s) {
            rho[t] += charge * ((double)s * kWeightUnit);
            sum[t] = 0ull;
        }
    }
}

int blocks(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return b < 1 ? 1 : (int)b;
}

}  // namespace
}  // namespace ohpic

extern "C" int ohpic_scatter_noalloc(const double *x, const double *y, const double *z, int64_t n, double charge,
                                     int32_t nx, int32_t ny, int32_t nz, int32_t weights, double *rho, void *stream)
{
    using namespace ohpic;
    if (n < 0 || nx < 1 || ny < 1 || nz < 1 || !rho || !isfinite(charge)) return OHPIC_ERR_INVALID;
    if (n > 0 && (!x || !y || !z)) return OHPIC_ERR_INVALID;
    if (weights != OHPIC_WEIGHTS_REFERENCE && weights != OHPIC_WEIGHTS_STANDARD) return OHPIC_ERR_INVALID;
    const int64_t ncell = (int64_t)nx * ny * nz;
    if (ncell > kNoAllocMaxNodes) return OHPIC_ERR_CAPACITY;   // grid larger than the static scratch
    // The scratch array's device address in the current device's context, looked
    // up on every call (it allocates nothing): a cached address would go stale if
    // the caller reset the device or tore down its primary context, after which
    // the module is loaded again and the array may move.
    void *addr = nullptr;
    if (cudaGetSymbolAddress(&addr, g_noalloc_sum) != cudaSuccess || !addr) {
        cudaGetLastError();
        return OHPIC_ERR_CUDA;
    }
    unsigned long long *sum = (unsigned long long *)addr;
    cudaStream_t s = (cudaStream_t)stream;
    if (n > 0) k_noalloc_deposit<<<blocks(n), 256, 0, s>>>(x, y, z, n, nx, ny, nz, weights, sum);
    k_noalloc_finish<<<blocks(ncell), 256, 0, s>>>(sum, ncell, charge, rho);
    return cudaGetLastError() == cudaSuccess ? OHPIC_OK : OHPIC_ERR_CUDA;
}
