// Tiled complex GEMM engine on the CUDA cores (FP64 for the plain path, FP32 storage
// variant for small mixed-precision helpers).
//
//   C(i, j) = sum_k a(i, k) * b(j, k)      i < M, j < N, k < K
//
// a(i,k) and b(j,k) are functors (they apply conjugation, phases, weights and
// bounds), the epilogue functor receives every computed element.  The loader
// mapping is selectable per operand so that the global reads coalesce whichever
// index is contiguous in memory: IMAJOR = consecutive threads read consecutive i
// (column-major with i the row), KMAJOR = consecutive threads read consecutive k.
//
// Tile 64 x 64, BK = 8, 256 threads, 4 x 4 complex accumulators per thread.
#pragma once
#include "cvec.cuh"
#include "forge_internal.cuh"

namespace forge {

enum LoadMajor { IMAJOR = 0, KMAJOR = 1 };

constexpr int ZG_BM = 64, ZG_BN = 64, ZG_BK = 8, ZG_THREADS = 256;

template <int MAJOR, int BROWS, class V, class F>
__device__ __forceinline__ void zg_load_tile(V (*S)[BROWS + 1], const F& f, int64_t r0, int64_t k0) {
    // loads BROWS x ZG_BK elements f(r0 + r, k0 + kk) into S[kk][r]
    constexpr int TOTAL = BROWS * ZG_BK;
#pragma unroll
    for (int q = 0; q < TOTAL / ZG_THREADS; ++q) {
        int idx = threadIdx.x + q * ZG_THREADS;
        int r, kk;
        if (MAJOR == IMAJOR) {
            r = idx % BROWS;
            kk = idx / BROWS;
        } else {
            kk = idx % ZG_BK;
            r = idx / ZG_BK;
        }
        S[kk][r] = f(r0 + r, k0 + kk);
    }
}

// Grid: x = tiles along M, y = tiles along N, z = batch (passed to the functors as blockIdx.z).
// LOWER: skip tiles entirely above the diagonal (i < j for all elements) and elements i < j.
template <class V, int AMAJOR, int BMAJOR, bool LOWER, class FA, class FB, class EPI>
__global__ void __launch_bounds__(ZG_THREADS) k_zgemm(int64_t M, int64_t N, int64_t K, FA fa, FB fb, EPI epi) {
    const int64_t i0 = (int64_t)blockIdx.x * ZG_BM, j0 = (int64_t)blockIdx.y * ZG_BN;
    if (LOWER && i0 + ZG_BM - 1 < j0) return;
    __shared__ V As[ZG_BK][ZG_BM + 1];
    __shared__ V Bs[ZG_BK][ZG_BN + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    V acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = vzero<V>();
    for (int64_t k0 = 0; k0 < K; k0 += ZG_BK) {
        zg_load_tile<AMAJOR, ZG_BM>(As, fa, i0, k0);
        zg_load_tile<BMAJOR, ZG_BN>(Bs, fb, j0, k0);
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < ZG_BK; ++kk) {
            V av[4], bv[4];
#pragma unroll
            for (int a = 0; a < 4; ++a) av[a] = As[kk][tx + 16 * a];
#pragma unroll
            for (int b = 0; b < 4; ++b) bv[b] = Bs[kk][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    acc[a][b].x = fma(av[a].x, bv[b].x, acc[a][b].x);
                    acc[a][b].x = fma(-av[a].y, bv[b].y, acc[a][b].x);
                    acc[a][b].y = fma(av[a].x, bv[b].y, acc[a][b].y);
                    acc[a][b].y = fma(av[a].y, bv[b].x, acc[a][b].y);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            int64_t i = i0 + tx + 16 * a, j = j0 + ty + 16 * b;
            if (i < M && j < N && (!LOWER || i >= j)) epi(i, j, acc[a][b]);
        }
}

template <class V, int AMAJOR, int BMAJOR, bool LOWER, class FA, class FB, class EPI>
inline int zgemm_launch(cudaStream_t st, int64_t M, int64_t N, int64_t K, int64_t batch, const FA& fa,
                        const FB& fb, const EPI& epi) {
    if (M <= 0 || N <= 0 || batch <= 0) return 0;
    dim3 grd((unsigned)((M + ZG_BM - 1) / ZG_BM), (unsigned)((N + ZG_BN - 1) / ZG_BN), (unsigned)batch);
    k_zgemm<V, AMAJOR, BMAJOR, LOWER><<<grd, ZG_THREADS, 0, st>>>(M, N, K, fa, fb, epi);
    FORGE_LAUNCH_CHECK();
    return 0;
}

}  // namespace forge
