// poisson_bc.cu -- the field solve on a bounded block with per-axis boundary kinds.
//
// Reference path (one rank, block = global block 0..n per axis):
//   new_PoissonFieldSolver / solve     src/field_solver/poisson_field_solver.f90:34-175
//   poissonSolver3d_solve              src/field_solver/poisson/poisson_solver3d.f90:134-207
//   wave-number table, wall terms      poisson_solver3d.f90:56-78, 81-102, 104-132
//   r2r kinds, logical ranges, norms   src/field_solver/fft/fftw3/mpi_fftw3_solver.f90:151-207, 235
//   boundary kinds                     src/field_solver/field_boundary_type.f90:21-71
//
// The reference runs FFTW's real-to-real transforms per axis: R2HC/HC2R on a
// periodic axis, DST-I on a Dirichlet one, DCT-I on a Neumann one, and DST-III /
// DST-II or DCT-III / DCT-II on the two mixed kinds.  cuFFT has no real-to-real
// transforms, so each one is a complex DFT of a symmetric extension of the line,
// with the extension and the output twiddles done by our own kernels:
//   DCT-I  (L points):  DFT of length 2(L-1) of the even extension,  Y_k = Z_k
//   DST-I  (L points):  DFT of length 2(L+1) of the odd extension,   Y_k = i Z_{k+1}
//   DCT-II:             DFT of length 2L of x_0..x_{L-1}, x_{L-1}..x_0,  Y_k = e^{-i pi k/2L} Z_k
//   DCT-III:            DFT of length 2L of u_m e^{-i pi m/2L} (u: x_0, x_1.., 0, -x_{L-1}.., -x_1)
//   DST-II:             DCT-II of (-1)^j x_j, read in reverse order
//   DST-III:            (-1)^k DCT-III of the reversed line
//   R2HC:               DFT of length L, split into the two real lines' spectra
//                       (F_A = (Z_k + conj Z_{L-k}) / 2, F_B = (Z_k - conj Z_{L-k}) / 2i)
//                       and stored half-complex (Re F_k at k <= L/2, Im F_k at L-k)
//   HC2R:               the two half-complex lines combined into G = F_A + i F_B,
//                       inverse DFT of length L: its real part is line A's, its
//                       imaginary part line B's.
// Two real lines per complex transform.  The working array R is real, and every
// transform above maps a real line to a real line and is linear, so one complex
// transform carries two lines: line A in the real part and line B, its partner
// half a block away along another axis (the pack axis), in the imaginary part.
// The DCT/DST forms are complex-linear as they stand; R2HC and HC2R separate and
// combine the pair explicitly.  Each pass therefore runs half the lines of
// cuFFT work and moves half the extension bytes of a complex working array.
// Every extension is stored line-contiguous, so cuFFT runs contiguous batched
// transforms on every axis; along y and z the extension and extraction kernels
// transpose 32 x 32 tiles through shared memory so that both their reads and
// their writes stay coalesced.
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <new>
#include <string>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

// The reference's pi literal (src/utils/science_constants.f90:4) for the tables.
constexpr double kRefPi = 3.14159265358979;

enum Xform { XF_R2HC, XF_HC2R, XF_DCT1, XF_DST1, XF_DCT2, XF_DCT3, XF_DST2, XF_DST3 };

struct Axis {
    int kind;        // OHPIC_BC_*
    int n;           // block nodes 0..n
    int L;           // logical points (transform length)
    int ls;          // global node of logical element 0
    int M;           // extension length
    int fwd, bwd;    // Xform
    double norm;     // mpi_fftw3_solver.f90:151-207
    bool wall_lo, wall_hi;
};

// convert_fft_type for the global block 0..n; false when the grid is too small.
bool make_axis(int kind, int n, Axis &a)
{
    a.kind = kind;
    a.n = n;
    a.wall_lo = a.wall_hi = false;
    switch (kind) {
    case OHPIC_BC_PERIODIC:
        a.fwd = XF_R2HC; a.bwd = XF_HC2R; a.ls = 0; a.L = n; a.M = a.L; a.norm = (double)a.L;
        break;
    case OHPIC_BC_DIRICHLET:
        a.fwd = a.bwd = XF_DST1; a.ls = 1; a.L = n - 1; a.M = 2 * (a.L + 1); a.norm = 2.0 * (a.L + 1.0);
        a.wall_lo = a.wall_hi = true;
        break;
    case OHPIC_BC_NEUMANN:
        a.fwd = a.bwd = XF_DCT1; a.ls = 0; a.L = n + 1; a.M = 2 * (a.L - 1); a.norm = 2.0 * (a.L - 1.0);
        break;
    case OHPIC_BC_DIRICHLET_NEUMANN:
        a.fwd = XF_DST3; a.bwd = XF_DST2; a.ls = 1; a.L = n; a.M = 2 * a.L; a.norm = 2.0 * a.L;
        a.wall_lo = true;
        break;
    case OHPIC_BC_NEUMANN_DIRICHLET:
        a.fwd = XF_DCT3; a.bwd = XF_DCT2; a.ls = 0; a.L = n; a.M = 2 * a.L; a.norm = 2.0 * a.L;
        a.wall_hi = true;
        break;
    default:
        return false;
    }
    return n >= 1 && a.L >= 1 && !(kind == OHPIC_BC_NEUMANN && a.L < 2);
}

// calc_wave_number (poisson_solver3d.f90:104-132), host code built without FMA
// contraction so the table has the reference's bits.
double wave_number(int k, int n, int kind)
{
    switch (kind) {
    case OHPIC_BC_PERIODIC:
        if (k <= n / 2) return 2.0 * sin(kRefPi * k / (double)n);
        return 2.0 * sin(kRefPi * (n - k) / (double)n);
    case OHPIC_BC_DIRICHLET: return 2.0 * (cos(kRefPi * (k + 1) / (double)(n + 1)) - 1.0);
    case OHPIC_BC_NEUMANN: return 2.0 * (cos(kRefPi * k / (double)n) - 1.0);
    default: return 2.0 * (cos(kRefPi * (k + 0.5) / (double)(n + 1)) - 1.0);
    }
}

// The negated eigenvalue of the 1-D Laplacian for logical mode i of each kind.
double eigenvalue(int i, int n, int kind)
{
    switch (kind) {
    case OHPIC_BC_PERIODIC: {
        const double w = wave_number(i, n, kind);
        return w * w;
    }
    case OHPIC_BC_DIRICHLET: return 2.0 - 2.0 * cos(kRefPi * (i + 1) / (double)n);
    case OHPIC_BC_NEUMANN: return 2.0 - 2.0 * cos(kRefPi * i / (double)n);
    default: return 2.0 - 2.0 * cos(kRefPi * (i + 0.5) / (double)n);
    }
}

// Lines of one axis of the real (L0, L1, L2) array R, x fastest, in pairs: the
// packed extents P equal L except along the pack axis, where P = H = ceil(L / 2)
// and the element at pack coordinate c is paired with the one at c + H (none
// when c + H is past the end: its half of the pair is zero and not stored).
// Lines are numbered over the packed extents of the two other axes, the lower
// axis fastest, so consecutive lines are consecutive in memory along y and z.
struct Lines {
    int axis, pack;
    int P0, P1, P2;          // packed extents
    int L0, L1;              // R's x and y extents (its strides)
    int H, Lp;               // pack offset and R's extent along the pack axis
    int64_t pstride;         // R distance from an element to its partner
    int64_t lines;
    int M;
};

// R index of element j of line `line` (the pair's first half); pair: the
// partner exists.
__device__ __forceinline__ int64_t r_index(const Lines &m, int64_t line, int j, bool &pair)
{
    int64_t c0, c1, c2;
    if (m.axis == 0) {
        c0 = j; c1 = line % m.P1; c2 = line / m.P1;
    } else if (m.axis == 1) {
        c0 = line % m.P0; c1 = j; c2 = line / m.P0;
    } else {
        c0 = line % m.P0; c1 = line / m.P0; c2 = j;
    }
    const int64_t cp = m.pack == 0 ? c0 : (m.pack == 1 ? c1 : c2);
    pair = cp + m.H < m.Lp;
    return c0 + (int64_t)m.L0 * (c1 + (int64_t)m.L1 * c2);
}

// Element j of line `line` as a complex pair (line A, line B).
__device__ __forceinline__ double2 load_pair(const Lines &m, const double *R, int64_t line, int j)
{
    bool pair;
    const int64_t i = r_index(m, line, j, pair);
    return make_double2(R[i], pair ? R[i + m.pstride] : 0.0);
}

__device__ __forceinline__ void store_pair(const Lines &m, double *R, int64_t line, int j, double2 v)
{
    bool pair;
    const int64_t i = r_index(m, line, j, pair);
    R[i] = v.x;
    if (pair) R[i + m.pstride] = v.y;
}

// (a + ib) e^{-i pi num / den}
__device__ __forceinline__ double2 rotate(double2 v, double num, double den)
{
    double s, c;
    sincospi(num / den, &s, &c);
    return make_double2(v.x * c + v.y * s, v.y * c - v.x * s);
}

// Extension element mi of line `line` for transform xf (see the header).
__device__ __forceinline__ double2 ext_value(const Lines &m, int xf, int L, const double *R, int64_t line, int mi)
{
    if (xf == XF_HC2R) {
        // G_k = F_A,k + i F_B,k from the half-complex pairs at k and L - k
        const int kk = mi == 0 ? 0 : L - mi;
        const double2 p = load_pair(m, R, line, mi);
        if (kk == mi) return p;   // k = 0, and k = L/2 for even L: real spectra
        const double2 q = load_pair(m, R, line, kk);
        return mi < kk ? make_double2(p.x - q.y, q.x + p.y) : make_double2(q.x + p.y, q.y - p.x);
    }
    int j = -1;
    double sgn = 1.0;
    bool twiddle = false;
    switch (xf) {
    case XF_R2HC: j = mi; break;
    case XF_DCT1: j = mi < L ? mi : m.M - mi; break;
    case XF_DST1:
        if (mi == 0 || mi == L + 1) j = -1;
        else if (mi <= L) j = mi - 1;
        else { j = m.M - mi - 1; sgn = -1.0; }
        break;
    case XF_DCT2: j = mi < L ? mi : 2 * L - 1 - mi; break;
    case XF_DST2:
        j = mi < L ? mi : 2 * L - 1 - mi;
        sgn = (j & 1) ? -1.0 : 1.0;
        break;
    default:   // DCT3, DST3 (the latter on the reversed line)
        if (mi == L) j = -1;
        else if (mi < L) j = mi;
        else { j = 2 * L - mi; sgn = -1.0; }
        if (xf == XF_DST3 && j >= 0) j = L - 1 - j;
        twiddle = true;
        break;
    }
    double2 v = make_double2(0.0, 0.0);
    if (j >= 0) {
        v = load_pair(m, R, line, j);
        v.x *= sgn;
        v.y *= sgn;
    }
    if (twiddle) v = rotate(v, (double)mi, 2.0 * L);
    return v;
}

// Output element k of line `line` from its transformed extension Z (= B + line * M).
__device__ __forceinline__ double2 extract_value(int xf, int L, const double2 *Z, int k)
{
    switch (xf) {
    case XF_DST1: {
        const double2 z = Z[k + 1];
        return make_double2(-z.y, z.x);
    }
    case XF_DCT2: return rotate(Z[k], (double)k, 2.0 * L);
    case XF_DST2: {
        const int kk = L - 1 - k;
        return rotate(Z[kk], (double)kk, 2.0 * L);
    }
    case XF_DST3: {
        const double2 z = Z[k];
        return (k & 1) ? make_double2(-z.x, -z.y) : z;
    }
    case XF_R2HC: {
        // the pair's spectra at k and L - k, stored half-complex
        const int kk = k == 0 ? 0 : L - k;
        const double2 z = Z[k], w = Z[kk];
        if (k <= kk) return make_double2(0.5 * (z.x + w.x), 0.5 * (z.y + w.y));   // Re F_A,k, Re F_B,k
        return make_double2(0.5 * (w.y - z.y), 0.5 * (z.x - w.x));               // Im F_A,L-k, Im F_B,L-k
    }
    default: return Z[k];   // HC2R, DCT1, DCT3
    }
}

// Every extension is stored line-contiguous, B[line * M + mi], so one batched
// cuFFT plan of contiguous transforms serves every axis.  Along x the lines of R
// are contiguous too and a thread per (line, mi) reads and writes coalesced.
// Along y and z consecutive lines are consecutive in R instead, so 32 x 32
// tiles go through shared memory: reads run along lines, writes along mi.
constexpr int kTile = 32, kTileRows = 8;

__global__ void k_extend_x(Lines m, int xf, int L, const double *R, double2 *B)
{
    const int64_t total = (int64_t)m.M * m.lines;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t line = t / m.M;
        const int mi = (int)(t - line * m.M);
        B[t] = ext_value(m, xf, L, R, line, mi);
    }
}

__global__ void k_extract_x(Lines m, int xf, int L, const double2 *B, double *R)
{
    const int64_t total = (int64_t)L * m.lines;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t line = t / L;
        const int k = (int)(t - line * L);
        store_pair(m, R, line, k, extract_value(xf, L, B + line * m.M, k));
    }
}

// grid (ceil(lines / 32), ceil(M / 32)), block (32, 8)
__global__ void k_extend_yz(Lines m, int xf, int L, const double *R, double2 *B)
{
    __shared__ double2 tile[kTile][kTile + 1];
    const int64_t l0 = (int64_t)blockIdx.x * kTile;
    const int m0 = blockIdx.y * kTile;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < kTile; r += kTileRows) {
        const int64_t line = l0 + tx;
        const int mi = m0 + r;
        if (line < m.lines && mi < m.M) tile[r][tx] = ext_value(m, xf, L, R, line, mi);
    }
    __syncthreads();
    for (int r = ty; r < kTile; r += kTileRows) {
        const int64_t line = l0 + r;
        const int mi = m0 + tx;
        if (line < m.lines && mi < m.M) B[line * m.M + mi] = tile[tx][r];
    }
}

// grid (ceil(lines / 32), ceil(L / 32)), block (32, 8)
__global__ void k_extract_yz(Lines m, int xf, int L, const double2 *B, double *R)
{
    __shared__ double2 tile[kTile][kTile + 1];
    const int64_t l0 = (int64_t)blockIdx.x * kTile;
    const int k0 = blockIdx.y * kTile;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int r = ty; r < kTile; r += kTileRows) {
        const int64_t line = l0 + r;
        const int k = k0 + tx;
        if (line < m.lines && k < L) tile[r][tx] = extract_value(xf, L, B + line * m.M, k);
    }
    __syncthreads();
    for (int r = ty; r < kTile; r += kTileRows) {
        const int64_t line = l0 + tx;
        const int k = k0 + r;
        if (line < m.lines && k < L) store_pair(m, R, line, k, tile[tx][r]);
    }
}

// Block-node geometry and the wall terms (poisson_solver3d.f90:156-168).
struct Block {
    int n[3], ls[3], L[3];
    int term_node_lo[3], term_node_hi[3];   // -1: no term
    double term_lo[3], term_hi[3];
    int kind[3];
    bool wall_lo[3], wall_hi[3];
    double wall_value_lo[3], wall_value_hi[3];
    bool zero_first;        // as written: element (0,0,0) of the block is in the transform
    double norm;            // product of the normalisers
};

__device__ __forceinline__ int64_t block_index(const Block &b, int i, int j, int k)
{
    return i + (int64_t)(b.n[0] + 1) * (j + (int64_t)(b.n[1] + 1) * k);
}

// phi = rho + wall terms on the logical range.
__global__ void k_pack(Block b, const double *rho, double *R)
{
    const int64_t total = (int64_t)b.L[0] * b.L[1] * b.L[2];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % b.L[0]);
        const int j = (int)((t / b.L[0]) % b.L[1]);
        const int k = (int)(t / ((int64_t)b.L[0] * b.L[1]));
        const int g[3] = {i + b.ls[0], j + b.ls[1], k + b.ls[2]};
        double v = rho[block_index(b, g[0], g[1], g[2])];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            if (g[d] == b.term_node_lo[d]) v += b.term_lo[d];
            if (g[d] == b.term_node_hi[d]) v += b.term_hi[d];
        }
        R[t] = v;
    }
}

// Division by the table (sum of three per-axis terms, added x, y, then z).
__global__ void k_divide(Block b, const double *tx, const double *ty, const double *tz, double *R)
{
    const int64_t total = (int64_t)b.L[0] * b.L[1] * b.L[2];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % b.L[0]);
        const int j = (int)((t / b.L[0]) % b.L[1]);
        const int k = (int)(t / ((int64_t)b.L[0] * b.L[1]));
        const double den = (tx[i] + ty[j]) + tz[k];
        R[t] = den == 0.0 || (b.zero_first && t == 0) ? 0.0 : R[t] / den;
    }
}

// phi on every block node: the transform's nodes scaled by the normalisers, a
// periodic axis' node n as the image of node 0, a Dirichlet wall its value.
__global__ void k_unpack(Block b, const double *R, double *phi)
{
    const int B0 = b.n[0] + 1, B1 = b.n[1] + 1;
    const int64_t total = (int64_t)B0 * B1 * (b.n[2] + 1);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int g[3] = {(int)(t % B0), (int)((t / B0) % B1), (int)(t / ((int64_t)B0 * B1))};
        bool wall = false;
        double v = 0.0;
        for (int d = 0; d < 3 && !wall; ++d) {
            if (b.kind[d] == OHPIC_BC_PERIODIC && g[d] == b.n[d]) {
                g[d] = 0;
            } else if (b.wall_lo[d] && g[d] == 0) {
                wall = true;
                v = b.wall_value_lo[d];
            } else if (b.wall_hi[d] && g[d] == b.n[d]) {
                wall = true;
                v = b.wall_value_hi[d];
            }
        }
        if (!wall) {
            const int64_t at = (g[0] - b.ls[0]) + (int64_t)b.L[0] * ((g[1] - b.ls[1]) + (int64_t)b.L[1] * (g[2] - b.ls[2]));
            v = R[at] / b.norm;
        }
        phi[t] = v;
    }
}

// E = -grad phi: the reference's central difference 0.5*((phi[i-1] - phi[i]) +
// (phi[i] - phi[i+1])) (poisson_field_solver.f90:139-144,165-170), wrapped on a
// periodic axis, one-sided at a wall of the other kinds.
__global__ void k_efield(Block b, const double *phi, double *e)
{
    const int B0 = b.n[0] + 1, B1 = b.n[1] + 1;
    const int64_t total = (int64_t)B0 * B1 * (b.n[2] + 1);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int g[3] = {(int)(t % B0), (int)((t / B0) % B1), (int)(t / ((int64_t)B0 * B1))};
        const double p0 = phi[t];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            int gm[3] = {g[0], g[1], g[2]}, gp[3] = {g[0], g[1], g[2]};
            double v;
            const int n = b.n[d];
            if (b.kind[d] == OHPIC_BC_PERIODIC) {
                const int c = g[d] == n ? 0 : g[d];
                gm[d] = c == 0 ? n - 1 : c - 1;
                gp[d] = c + 1 == n ? 0 : c + 1;
                v = 0.5 * ((phi[block_index(b, gm[0], gm[1], gm[2])] - p0) + (p0 - phi[block_index(b, gp[0], gp[1], gp[2])]));
            } else if (g[d] == 0) {
                gp[d] = 1;
                v = p0 - phi[block_index(b, gp[0], gp[1], gp[2])];
            } else if (g[d] == n) {
                gm[d] = n - 1;
                v = phi[block_index(b, gm[0], gm[1], gm[2])] - p0;
            } else {
                gm[d] = g[d] - 1;
                gp[d] = g[d] + 1;
                v = 0.5 * ((phi[block_index(b, gm[0], gm[1], gm[2])] - p0) + (p0 - phi[block_index(b, gp[0], gp[1], gp[2])]));
            }
            e[(int64_t)d * total + t] = v;
        }
    }
}

int grid_of(int64_t n)
{
    int64_t b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return b < 1 ? 1 : (int)b;
}

}  // namespace
}  // namespace ohpic

using namespace ohpic;

struct ohpic_poisson {
    int dev = 0;
    Axis ax[3];
    Block blk;
    Lines lines[3];
    cufftHandle plan[3] = {0, 0, 0};
    bool planned[3] = {false, false, false};
    double *R = nullptr;
    double2 *B = nullptr;
    double *table[3] = {nullptr, nullptr, nullptr};
    double *rho = nullptr, *phi = nullptr, *e = nullptr;   // device staging of the host entry point
    cudaStream_t stream = nullptr;
    int64_t nodes = 0;
    std::string err;
};

namespace {

int pfail(ohpic_poisson *p, int code, const std::string &msg)
{
    if (p) p->err = msg;
    return code;
}

void release(ohpic_poisson *p)
{
    cudaSetDevice(p->dev);
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (int d = 0; d < 3; ++d) {
        if (p->planned[d]) cufftDestroy(p->plan[d]);
        if (p->table[d]) cudaFree(p->table[d]);
    }
    for (void *q : {(void *)p->R, (void *)p->B, (void *)p->rho, (void *)p->phi, (void *)p->e})
        if (q) cudaFree(q);
    if (p->stream) cudaStreamDestroy(p->stream);
}

// forward or backward transform along one axis of p->R
int transform(ohpic_poisson *p, int d, int xf, cudaStream_t st)
{
    const Lines &m = p->lines[d];
    const int L = p->ax[d].L;
    const unsigned lt = (unsigned)((m.lines + kTile - 1) / kTile);
    if (d == 0)
        k_extend_x<<<grid_of((int64_t)m.M * m.lines), 256, 0, st>>>(m, xf, L, p->R, p->B);
    else
        k_extend_yz<<<dim3(lt, (unsigned)((m.M + kTile - 1) / kTile)), dim3(kTile, kTileRows), 0, st>>>(m, xf, L, p->R,
                                                                                                      p->B);
    if (cufftSetStream(p->plan[d], st) != CUFFT_SUCCESS)
        return pfail(p, OHPIC_ERR_CUDA, "cufftSetStream failed");
    const int dir = xf == XF_HC2R ? CUFFT_INVERSE : CUFFT_FORWARD;
    const cufftResult r = cufftExecZ2Z(p->plan[d], (cufftDoubleComplex *)p->B, (cufftDoubleComplex *)p->B, dir);
    if (r != CUFFT_SUCCESS) return pfail(p, OHPIC_ERR_CUDA, "cufftExecZ2Z failed (" + std::to_string((int)r) + ")");
    if (d == 0)
        k_extract_x<<<grid_of((int64_t)L * m.lines), 256, 0, st>>>(m, xf, L, p->B, p->R);
    else
        k_extract_yz<<<dim3(lt, (unsigned)((L + kTile - 1) / kTile)), dim3(kTile, kTileRows), 0, st>>>(m, xf, L, p->B,
                                                                                                     p->R);
    return OHPIC_OK;
}

}  // namespace

extern "C" {

int ohpic_poisson_create(const int32_t n[3], const int32_t kinds[3], const double boundary_values[6], int32_t table,
                         int32_t device, ohpic_poisson **out)
{
    if (!n || !kinds || !out) return OHPIC_ERR_INVALID;
    *out = nullptr;
    if (table != OHPIC_TABLE_AS_WRITTEN && table != OHPIC_TABLE_CORRECTED) return OHPIC_ERR_INVALID;
    const double zero[6] = {0, 0, 0, 0, 0, 0};
    const double *bv = boundary_values ? boundary_values : zero;
    for (int k = 0; k < 6; ++k)
        if (!std::isfinite(bv[k])) return OHPIC_ERR_INVALID;
    ohpic_poisson *p = new (std::nothrow) ohpic_poisson();
    if (!p) return OHPIC_ERR_OOM;
    for (int d = 0; d < 3; ++d)
        if (n[d] > 4096 || !make_axis(kinds[d], n[d], p->ax[d])) {
            delete p;
            return OHPIC_ERR_INVALID;
        }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        delete p;
        return OHPIC_ERR_CUDA;
    }
    p->dev = device;
    cudaSetDevice(device);
    const bool corrected = table == OHPIC_TABLE_CORRECTED;
    Block &b = p->blk;
    b.norm = 1.0;
    bool all_start0 = true;
    for (int d = 0; d < 3; ++d) {
        const Axis &a = p->ax[d];
        b.n[d] = a.n;
        b.ls[d] = a.ls;
        b.L[d] = a.L;
        b.kind[d] = a.kind;
        b.wall_lo[d] = a.wall_lo;
        b.wall_hi[d] = a.wall_hi;
        b.wall_value_lo[d] = corrected ? bv[2 * d] : 0.0;
        b.wall_value_hi[d] = corrected ? bv[2 * d + 1] : 0.0;
        all_start0 = all_start0 && a.ls == 0;
        // calc_boundary_term (poisson_solver3d.f90:81-102), on the block's first and
        // last node planes as written; corrected, a Dirichlet wall's potential enters
        // the adjacent interior node and a periodic axis takes no term.
        double t0, t1;
        switch (a.kind) {
        case OHPIC_BC_PERIODIC: t0 = bv[2 * d]; t1 = bv[2 * d + 1]; break;
        case OHPIC_BC_DIRICHLET: t0 = -bv[2 * d]; t1 = -bv[2 * d + 1]; break;
        case OHPIC_BC_NEUMANN: t0 = 2.0 * bv[2 * d]; t1 = -2.0 * bv[2 * d + 1]; break;
        default: t0 = -bv[2 * d]; t1 = -2.0 * bv[2 * d + 1]; break;
        }
        int lo = 0, hi = a.n;
        if (corrected) {
            if (a.kind == OHPIC_BC_PERIODIC) {
                lo = hi = -1;
                t0 = t1 = 0.0;
            } else {
                if (a.wall_lo) { t0 = bv[2 * d]; lo = 1; }
                else t0 = 2.0 * bv[2 * d];
                if (a.wall_hi) { t1 = bv[2 * d + 1]; hi = a.n - 1; }
                else t1 = -2.0 * bv[2 * d + 1];
            }
        }
        b.term_node_lo[d] = lo;
        b.term_node_hi[d] = hi;
        b.term_lo[d] = t0;
        b.term_hi[d] = t1;
    }
    b.norm = p->ax[0].norm * p->ax[1].norm * p->ax[2].norm;
    b.zero_first = !corrected && all_start0;
    p->nodes = (int64_t)(n[0] + 1) * (n[1] + 1) * (n[2] + 1);
    const int64_t nl = (int64_t)b.L[0] * b.L[1] * b.L[2];
    int64_t maxb = 0;
    for (int d = 0; d < 3; ++d) {
        // pair along the longer of the two other axes (the slower one on a tie)
        Lines &m = p->lines[d];
        const int u = d == 0 ? 1 : 0, v = d == 2 ? 1 : 2;
        const int pk = b.L[u] > b.L[v] ? u : v;
        const int H = (b.L[pk] + 1) / 2;
        int P[3] = {b.L[0], b.L[1], b.L[2]};
        P[pk] = H;
        m.axis = d;
        m.pack = pk;
        m.P0 = P[0];
        m.P1 = P[1];
        m.P2 = P[2];
        m.L0 = b.L[0];
        m.L1 = b.L[1];
        m.H = H;
        m.Lp = b.L[pk];
        m.pstride = (int64_t)H * (pk == 0 ? 1 : (pk == 1 ? (int64_t)b.L[0] : (int64_t)b.L[0] * b.L[1]));
        m.lines = (int64_t)P[0] * P[1] * P[2] / P[d];
        m.M = p->ax[d].M;
        maxb = std::max<int64_t>(maxb, (int64_t)m.M * m.lines);
    }
    int rc = OHPIC_OK;
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) rc = OHPIC_ERR_CUDA;
    if (rc == OHPIC_OK && (cudaMalloc((void **)&p->R, sizeof(double) * nl) != cudaSuccess ||
                           cudaMalloc((void **)&p->B, sizeof(double2) * maxb) != cudaSuccess))
        rc = pfail(p, OHPIC_ERR_OOM, "poisson: device buffers");
    for (int d = 0; d < 3 && rc == OHPIC_OK; ++d) {
        // the table per axis: squared wave numbers at the element's global node (as
        // written, poisson_solver3d.f90:62-78) or the Laplacian's eigenvalues
        const Axis &a = p->ax[d];
        std::string host(sizeof(double) * a.L, '\0');
        double *h = (double *)&host[0];
        for (int i = 0; i < a.L; ++i) {
            if (corrected) {
                h[i] = eigenvalue(i, a.n, a.kind);
            } else {
                const double w = wave_number(i + a.ls, a.n, a.kind);
                h[i] = w * w;
            }
        }
        if (cudaMalloc((void **)&p->table[d], sizeof(double) * a.L) != cudaSuccess ||
            cudaMemcpy(p->table[d], h, sizeof(double) * a.L, cudaMemcpyHostToDevice) != cudaSuccess) {
            rc = pfail(p, OHPIC_ERR_OOM, "poisson: table");
            break;
        }
        const Lines &m = p->lines[d];
        int len = m.M, emb = m.M;
        const cufftResult r = cufftPlanMany(&p->plan[d], 1, &len, &emb, 1, m.M, &emb, 1, m.M, CUFFT_Z2Z, (int)m.lines);
        if (r != CUFFT_SUCCESS) {
            rc = pfail(p, OHPIC_ERR_CUDA, "cufftPlanMany failed (" + std::to_string((int)r) + ")");
            break;
        }
        p->planned[d] = true;
    }
    if (rc != OHPIC_OK) {
        release(p);
        delete p;
        return rc;
    }
    *out = p;
    return OHPIC_OK;
}

int ohpic_poisson_destroy(ohpic_poisson *p)
{
    if (!p) return OHPIC_OK;
    release(p);
    delete p;
    return OHPIC_OK;
}

int ohpic_poisson_solve_device(ohpic_poisson *p, const double *rho, double *phi, double *e, void *stream)
{
    if (!p || !rho || !phi) return pfail(p, OHPIC_ERR_INVALID, "poisson: null rho or phi");
    cudaSetDevice(p->dev);
    cudaStream_t st = (cudaStream_t)stream;
    const Block &b = p->blk;
    const int64_t nl = (int64_t)b.L[0] * b.L[1] * b.L[2];
    k_pack<<<grid_of(nl), 256, 0, st>>>(b, rho, p->R);
    for (int d = 0; d < 3; ++d) {
        const int rc = transform(p, d, p->ax[d].fwd, st);
        if (rc != OHPIC_OK) return rc;
    }
    k_divide<<<grid_of(nl), 256, 0, st>>>(b, p->table[0], p->table[1], p->table[2], p->R);
    for (int d = 2; d >= 0; --d) {
        const int rc = transform(p, d, p->ax[d].bwd, st);
        if (rc != OHPIC_OK) return rc;
    }
    k_unpack<<<grid_of(p->nodes), 256, 0, st>>>(b, p->R, phi);
    if (e) k_efield<<<grid_of(p->nodes), 256, 0, st>>>(b, phi, e);
    const cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) return pfail(p, OHPIC_ERR_CUDA, std::string("poisson: ") + cudaGetErrorString(ce));
    return OHPIC_OK;
}

int ohpic_poisson_solve(ohpic_poisson *p, const double *rho, double *phi, double *e)
{
    if (!p || !rho || !phi) return pfail(p, OHPIC_ERR_INVALID, "poisson: null rho or phi");
    cudaSetDevice(p->dev);
    const size_t bytes = sizeof(double) * (size_t)p->nodes;
    if (!p->rho && (cudaMalloc((void **)&p->rho, bytes) != cudaSuccess ||
                    cudaMalloc((void **)&p->phi, bytes) != cudaSuccess)) {
        cudaGetLastError();
        return pfail(p, OHPIC_ERR_OOM, "poisson: staging");
    }
    if (e && !p->e && cudaMalloc((void **)&p->e, 3 * bytes) != cudaSuccess) {
        cudaGetLastError();
        return pfail(p, OHPIC_ERR_OOM, "poisson: staging");
    }
    if (cudaMemcpyAsync(p->rho, rho, bytes, cudaMemcpyHostToDevice, p->stream) != cudaSuccess)
        return pfail(p, OHPIC_ERR_CUDA, "poisson: rho copy");
    int rc = ohpic_poisson_solve_device(p, p->rho, p->phi, e ? p->e : nullptr, p->stream);
    if (rc != OHPIC_OK) return rc;
    if (cudaMemcpyAsync(phi, p->phi, bytes, cudaMemcpyDeviceToHost, p->stream) != cudaSuccess ||
        (e && cudaMemcpyAsync(e, p->e, 3 * bytes, cudaMemcpyDeviceToHost, p->stream) != cudaSuccess))
        return pfail(p, OHPIC_ERR_CUDA, "poisson: result copy");
    const cudaError_t ce = cudaStreamSynchronize(p->stream);
    if (ce != cudaSuccess) return pfail(p, OHPIC_ERR_CUDA, std::string("poisson: ") + cudaGetErrorString(ce));
    return OHPIC_OK;
}

int ohpic_poisson_last_error(const ohpic_poisson *p, char *buf, size_t len)
{
    if (!p || !buf || len == 0) return OHPIC_ERR_INVALID;
    const size_t n = std::min(len - 1, p->err.size());
    memcpy(buf, p->err.data(), n);
    buf[n] = 0;
    return OHPIC_OK;
}

}  // extern "C"
