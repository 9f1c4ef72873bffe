// C-ABI check of the tcgen05 TF32 GEMM alone: D = A B^T (row-major, fp32), used by the
// GPU tests to validate the tensor-core path against an FP64 product.
#include "tc_gemm.cuh"

namespace forge {

struct StoreEpi {
    float* D;
    int64_t ldd, strideD;
    __device__ void operator()(int64_t b, int64_t row, int64_t col0, const float* v, int64_t M, int64_t N) const {
        if (row >= M) return;
        float* d = D + b * strideD + row * ldd;
#pragma unroll
        for (int q = 0; q < 32; ++q)
            if (col0 + q < N) d[col0 + q] = v[q];
    }
};

}  // namespace forge

using namespace forge;

static int selftest_run(int64_t M, int64_t N, int64_t K, int64_t batch, const float* A, const float* B, float* D,
                        TcFault flt) {
    if (M < 1 || N < 1 || K < 1 || batch < 1 || !A || !B || !D) {
        set_error(FORGE_ERR_ARG, "selftest_tc_gemm: bad arguments");
        return FORGE_ERR_ARG;
    }
    const int64_t ld = (K + 3) / 4 * 4;
    DevBuf dA, dB, dD, derr;
    int rc = 0;
    if ((rc = dA.ensure(batch * M * ld * 4)) || (rc = dB.ensure(batch * N * ld * 4)) ||
        (rc = dD.ensure(batch * M * N * 4)) || (rc = derr.ensure(sizeof(int))))
        return rc;
    cudaStream_t st;
    FORGE_CUDA(cudaStreamCreate(&st));
    FORGE_CUDA(cudaMemsetAsync(dA.ptr, 0, batch * M * ld * 4, st));
    FORGE_CUDA(cudaMemsetAsync(dB.ptr, 0, batch * N * ld * 4, st));
    FORGE_CUDA(cudaMemsetAsync(derr.ptr, 0, sizeof(int), st));
    FORGE_CUDA(cudaMemcpy2DAsync(dA.ptr, ld * 4, A, K * 4, K * 4, batch * M, cudaMemcpyHostToDevice, st));
    FORGE_CUDA(cudaMemcpy2DAsync(dB.ptr, ld * 4, B, K * 4, K * 4, batch * N, cudaMemcpyHostToDevice, st));
    TcOperand a{dA.as<float>(), M, K, ld, M * ld};
    TcOperand b{dB.as<float>(), N, K, ld, N * ld};
    rc = tc_gemm_tf32(st, a, b, K, batch, StoreEpi{dD.as<float>(), N, M * N}, derr.as<int>(), 0, flt);
    int herr = 0;
    if (!rc) {
        FORGE_CUDA(cudaMemcpyAsync(D, dD.ptr, batch * M * N * 4, cudaMemcpyDeviceToHost, st));
        FORGE_CUDA(cudaMemcpyAsync(&herr, derr.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
        FORGE_CUDA(cudaStreamSynchronize(st));
    }
    cudaStreamDestroy(st);
    if (!rc && herr) {
        set_error(FORGE_ERR_TIMEOUT, "tcgen05 GEMM: a bounded mbarrier wait gave up");
        rc = FORGE_ERR_TIMEOUT;
    }
    return rc;
}

extern "C" int forge_gpu_selftest_tc_gemm(int64_t M, int64_t N, int64_t K, int64_t batch, const float* A,
                                          const float* B, float* D) {
    return selftest_run(M, N, K, batch, A, B, D, TcFault{});
}

// Failure detection without a fault: the producer stops after K block 0, so the MMA issuer's
// bounded wait for block 1 runs out (spin_limit iterations); the kernel sets its error flag,
// drains, frees its TMEM and returns, and the call reports FORGE_ERR_TIMEOUT.
extern "C" int forge_gpu_selftest_tc_gemm_timeout(int64_t M, int64_t N, int64_t K, int64_t spin_limit,
                                                  const float* A, const float* B, float* D) {
    if (K <= 32 || spin_limit < 1 || spin_limit > (int64_t)TC_SPIN_LIMIT) {
        set_error(FORGE_ERR_ARG, "selftest_tc_gemm_timeout: needs K > 32 and 1 <= spin_limit <= %u", TC_SPIN_LIMIT);
        return FORGE_ERR_ARG;
    }
    TcFault f;
    f.spin_limit = (uint32_t)spin_limit;
    f.stop_loads_at = 1;
    return selftest_run(M, N, K, 1, A, B, D, f);
}
