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

// Grid: x = tiles along M (times K splits), y = tiles along N, z = batch (passed to the functors
// as blockIdx.z).  LOWER: skip tiles entirely above the diagonal and elements i < j.
// SPLIT: blockIdx.x = s * (M tiles) + tile; split s sums k in [s kchunk, min(K, (s+1) kchunk))
// (kchunk a multiple of ZG_BK, so no k is summed twice) and the epilogue is called as
// epi(s, i, j, c) with its partial sum.
template <class V, int AMAJOR, int BMAJOR, bool LOWER, bool SPLIT, class FA, class FB, class EPI>
__global__ void __launch_bounds__(ZG_THREADS)
    k_zgemm(int64_t M, int64_t N, int64_t K, int64_t kchunk, FA fa, FB fb, EPI epi) {
    const int64_t mt = (M + ZG_BM - 1) / ZG_BM;
    const int64_t split = SPLIT ? blockIdx.x / mt : 0;
    const int64_t i0 = (int64_t)(blockIdx.x - split * mt) * ZG_BM, j0 = (int64_t)blockIdx.y * ZG_BN;
    const int64_t klo = SPLIT ? split * kchunk : 0;
    const int64_t khi = SPLIT ? (K < klo + kchunk ? K : klo + kchunk) : K;
    if (LOWER && i0 + ZG_BM - 1 < j0) return;
    __shared__ V As[ZG_BK][ZG_BM + 1];
    __shared__ V Bs[ZG_BK][ZG_BN + 1];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    V acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = vzero<V>();
    for (int64_t k0 = klo; k0 < khi; k0 += ZG_BK) {
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
            if (i < M && j < N && (!LOWER || i >= j)) {
                if constexpr (SPLIT)
                    epi(split, i, j, acc[a][b]);
                else
                    epi(i, j, acc[a][b]);
            }
        }
}

template <class V, int AMAJOR, int BMAJOR, bool LOWER, class FA, class FB, class EPI>
inline int zgemm_launch(cudaStream_t st, int64_t M, int64_t N, int64_t K, int64_t batch, const FA& fa,
                        const FB& fb, const EPI& epi) {
    if (M <= 0 || N <= 0 || batch <= 0) return 0;
    dim3 grd((unsigned)((M + ZG_BM - 1) / ZG_BM), (unsigned)((N + ZG_BN - 1) / ZG_BN), (unsigned)batch);
    k_zgemm<V, AMAJOR, BMAJOR, LOWER, false><<<grd, ZG_THREADS, 0, st>>>(M, N, K, K, fa, fb, epi);
    FORGE_LAUNCH_CHECK();
    return 0;
}

// Number of K splits zgemm_launch_splitk runs for a K extent when `want` are asked for (none empty).
inline int64_t zg_ksplit_count(int64_t K, int64_t want) {
    if (want <= 1 || K <= ZG_BK) return 1;
    int64_t chunk = (K + want - 1) / want;
    chunk = (chunk + ZG_BK - 1) / ZG_BK * ZG_BK;
    return (K + chunk - 1) / chunk;
}

// Split-K form: ks = zg_ksplit_count(K, want) partial products, epilogue epi(s, i, j, c).
template <class V, int AMAJOR, int BMAJOR, class FA, class FB, class EPI>
inline int zgemm_launch_splitk(cudaStream_t st, int64_t M, int64_t N, int64_t K, int64_t batch, int64_t want,
                               const FA& fa, const FB& fb, const EPI& epi) {
    if (M <= 0 || N <= 0 || batch <= 0) return 0;
    const int64_t ks = zg_ksplit_count(K, want);
    int64_t chunk = (K + ks - 1) / ks;
    chunk = (chunk + ZG_BK - 1) / ZG_BK * ZG_BK;
    const int64_t mt = (M + ZG_BM - 1) / ZG_BM;
    dim3 grd((unsigned)(mt * ks), (unsigned)((N + ZG_BN - 1) / ZG_BN), (unsigned)batch);
    k_zgemm<V, AMAJOR, BMAJOR, false, true><<<grd, ZG_THREADS, 0, st>>>(M, N, K, chunk, fa, fb, epi);
    FORGE_LAUNCH_CHECK();
    return 0;
}

}  // namespace forge
