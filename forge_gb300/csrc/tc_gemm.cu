// Host helpers of the tcgen05 GEMM: TMA descriptors through the driver entry point
// (no link-time dependency on libcuda).
#include <cudaTypedefs.h>

#include <mutex>

#include "tc_gemm.cuh"

namespace forge {

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
static std::once_flag g_encode_once;

int tc_make_tmap(CUtensorMap* map, const TcOperand& op, int64_t batch, int box_rows) {
    std::call_once(g_encode_once, []() {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    });
    if (!g_encode) {
        set_error(FORGE_ERR_CUDA, "cuTensorMapEncodeTiled not available from the driver");
        return FORGE_ERR_CUDA;
    }
    const int64_t planes = op.nplanes > 0 ? op.nplanes : batch;
    const int64_t bstride = (planes > 1) ? op.batch_stride : op.rows * op.ld;
    cuuint64_t dims[3] = {(cuuint64_t)op.cols, (cuuint64_t)op.rows, (cuuint64_t)planes};
    cuuint64_t strides[2] = {(cuuint64_t)op.ld * 4, (cuuint64_t)bstride * 4};
    cuuint32_t box[3] = {(cuuint32_t)TC_BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)op.ptr, dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error(FORGE_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) rows=%lld cols=%lld ld=%lld", (int)r,
                  (long long)op.rows, (long long)op.cols, (long long)op.ld);
        return FORGE_ERR_CUDA;
    }
    return 0;
}

}  // namespace forge
