// kcna_tmap.cu - TMA tensor map of the BF16 rows for the Gram-tile kernels.
//
// The rows are a 2-D tensor (ld elements x n rows, BF16, row pitch 2*ld
// bytes).  The map's box is 64 elements x 1 row with 128-byte swizzle, the
// shape tile::gather4 loads use: four rows of one 64-element K block land as
// 4 x 128 bytes in the swizzled K-major layout the MMA descriptors read;
// columns beyond ld read as zero.
#include <cuda.h>

#include "kcna_internal.h"

namespace {
typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
}

kcna_status kcna_rows_tmap(kcna_ctx *c, void *out128) {
    static EncodeTiled encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return kcna_fail(c, KCNA_E_CUDA, "cuTensorMapEncodeTiled not available");
        encode = reinterpret_cast<EncodeTiled>(fn);
    }
    if (!c->Xh || (c->ld & 7u)) return kcna_fail(c, KCNA_E_STATE, "tensor map: no BF16 rows with 16-byte pitch");
    const cuuint64_t dims[2] = {c->ld, c->n_total};
    const cuuint64_t strides[1] = {(cuuint64_t)c->ld * 2};
    const cuuint32_t box[2] = {64, 1};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(reinterpret_cast<CUtensorMap *>(out128), CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, c->Xh, dims,
                        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? KCNA_OK : kcna_fail(c, KCNA_E_CUDA, "cuTensorMapEncodeTiled failed");
}
