// tma_map.cu -- host-side tensor map of the padded E field for TMA staging.
//
// The map describes E as a 3-D tensor of reals {4*gx, gy, gz} (row pitch
// 4*gx reals, plane pitch 4*gx*gy reals) with a box of {4*sx, sy, sz}: the
// staged node box of one tile.  It is re-encoded whenever E is reallocated or
// the tile shape or halo changes.  cuTensorMapEncodeTiled is reached through
// cudaGetDriverEntryPointByVersion, so the library does not link libcuda.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include "ohpic_internal.cuh"

namespace ohpic {
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static bool looked = false;
    if (!looked) {
        looked = true;
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        else
            cudaGetLastError();
    }
    return fn;
}

}  // namespace

// Encodes (or keeps) the E map for the current layout; emap_ok is false when the
// driver offers no encoder, in which case the kernels stage E with plain loads.
void ensure_emap(ohpic_ctx *c)
{
    const Geom &g = c->g;
    if (c->emap_ok && c->emap_for == c->epad && c->emap_key[0] == g.sx && c->emap_key[1] == g.sy &&
        c->emap_key[2] == g.sz && c->emap_key[3] == g.gx)
        return;
    c->emap_ok = false;
    PFN_cuTensorMapEncodeTiled_v12000 enc = encode_fn();
    if (!enc) return;
    const bool f64 = c->cfg.precision == OHPIC_FP64;
    const cuuint64_t es = f64 ? 8 : 4;
    const cuuint64_t dims[3] = {(cuuint64_t)4 * g.gx, (cuuint64_t)g.gy, (cuuint64_t)g.gz};
    const cuuint64_t strides[2] = {(cuuint64_t)4 * g.gx * es, (cuuint64_t)4 * g.gx * g.gy * es};
    const cuuint32_t box[3] = {(cuuint32_t)(4 * g.sx), (cuuint32_t)g.sy, (cuuint32_t)g.sz};
    const cuuint32_t estr[3] = {1, 1, 1};
    if (box[0] > 256 || box[1] > 256 || box[2] > 256) return;
    CUresult r = enc(&c->emap, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, c->epad,
                     dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return;
    c->emap_ok = true;
    c->emap_for = c->epad;
    c->emap_key[0] = g.sx;
    c->emap_key[1] = g.sy;
    c->emap_key[2] = g.sz;
    c->emap_key[3] = g.gx;
}

}  // namespace ohpic
