// K5 on the tensor cores: C_k = conj(X) X^T over the occupied columns of X_k, accumulated with
// the integer Bloch phases into the four FP64 cells of P(R) (Solve, HartreeFock.f90:456-473).
//
// X_k is split into TF32 planes with orbital rows and band-contiguous K:
//   0 hi.re  1 hi.im  2 lo.re  3 lo.im  4 -hi.re  5 -lo.re
// Re C = Xr Xr^T + Xi Xi^T and Im C = Xr Xi^T - Xi Xr^T are two real GEMMs whose K runs over six
// plane segments (hi*hi + hi*lo + lo*hi for each product), so no operand is copied or negated
// per GEMM.  Only lower tiles are formed; the epilogue writes (i, j) and (j, i).
#include <vector>

#include "proj.cuh"
#include "tc_gemm.cuh"

namespace forge {

__device__ inline float tf32_hi_p(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// X (n x K columns of X_k, column-major, FP64) -> 6 planes (n rows x ldk, band contiguous).
// Also adds sum_k |X_ik|^2 of its 32 columns, in FP64, into diag[i]: the diagonal of C (the site
// densities, which drive the long-range Hartree potential) is taken from there, not from the
// tensor-core product.
__global__ void k_stage_proj(const double2* __restrict__ X, int64_t ldx, int64_t n, int64_t K, int64_t ldk,
                             float* __restrict__ Xt, double* __restrict__ diag) {
    __shared__ double2 tile[32][33];
    __shared__ double dpart[8][32];
    const int64_t i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    double dsum = 0.0;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int64_t i = i0 + threadIdx.x, k = k0 + q;
        const double2 x = (i < n && k < K) ? X[i + k * ldx] : make_double2(0.0, 0.0);
        tile[q][threadIdx.x] = x;
        dsum += x.x * x.x + x.y * x.y;
    }
    dpart[threadIdx.y][threadIdx.x] = dsum;
    __syncthreads();
    if (threadIdx.y == 0 && i0 + threadIdx.x < n) {
        double t = 0.0;
        for (int y = 0; y < (int)blockDim.y; ++y) t += dpart[y][threadIdx.x];
        atomicAdd(diag + i0 + threadIdx.x, t);
    }
    const size_t P = (size_t)n * ldk;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int64_t i = i0 + q, k = k0 + threadIdx.x;
        if (i < n && k < ldk) {
            const double2 x = tile[threadIdx.x][q];
            const float xr = (float)x.x, xi = (float)x.y;
            const float hr = tf32_hi_p(xr), hi = tf32_hi_p(xi);
            const float lr = (float)(x.x - (double)hr), li = (float)(x.y - (double)hi);
            const size_t o = (size_t)i * ldk + k;
            Xt[o] = hr;
            Xt[P + o] = hi;
            Xt[2 * P + o] = lr;
            Xt[3 * P + o] = li;
            Xt[4 * P + o] = -hr;
            Xt[5 * P + o] = -lr;
        }
    }
}

// GEMM epilogue: the lower triangle of Re C or Im C, plain coalesced stores (column-major n x n)
struct ProjStoreEpi {
    float* C;
    int64_t n;
    __device__ void operator()(int64_t b, int64_t row, int64_t col0, const float* v, int64_t M, int64_t N) const {
        (void)b;
        if (row >= M) return;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
            const int64_t j = col0 + q;
            if (j < N && j <= row) C[row + j * n] = v[q];
        }
    }
};

// P_c += ph_c C on tile (bi, bj) and P_c += ph_c conj(C) on the mirrored tile (bj, bi), for the
// Hermitian C of which only the lower triangle (Cr, Ci) was formed; 32 x 32 tiles, coalesced.
template <class CT>
__global__ void __launch_bounds__(256) k_proj_accum(double2* __restrict__ P, const CT* __restrict__ Cr,
                                                    const CT* __restrict__ Ci, const double* __restrict__ diag,
                                                    int64_t n, double2 ph0, double2 ph1, double2 ph2, double2 ph3) {
    const int64_t bi = blockIdx.x, bj = blockIdx.y;
    if (bi < bj) return;
    __shared__ CT sr[32][33], si[32][33];
    const int64_t i0 = bi * 32, j0 = bj * 32;
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int64_t i = i0 + threadIdx.x, j = j0 + y;
        const bool ok = i < n && j < n && i >= j;
        sr[y][threadIdx.x] = ok ? Cr[i + j * n] : (CT)0;                // sr[col][row]
        si[y][threadIdx.x] = (ok && i != j) ? Ci[i + j * n] : (CT)0;
    }
    __syncthreads();
    const double2 ph[4] = {ph0, ph1, ph2, ph3};
    const size_t NN = (size_t)n * n;
    // tile (bi, bj): element (i, j) = C(i, j) if i >= j else conj(C(j, i)) (diagonal tile only)
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int64_t i = i0 + threadIdx.x, j = j0 + y;
        if (i >= n || j >= n) continue;
        double cr, ci;
        if (i == j) {
            cr = diag[i];
            ci = 0.0;
        } else if (i > j) {
            cr = sr[y][threadIdx.x];
            ci = si[y][threadIdx.x];
        } else {
            cr = sr[threadIdx.x][y];
            ci = -si[threadIdx.x][y];
        }
        const size_t o = i + (size_t)j * n;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            double2 p = P[c * NN + o];
            p.x += ph[c].x * cr - ph[c].y * ci;
            p.y += ph[c].x * ci + ph[c].y * cr;
            P[c * NN + o] = p;
        }
    }
    if (bi == bj) return;
    // mirrored tile (bj, bi): element (j, i) = conj(C(i, j))
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int64_t j = j0 + threadIdx.x, i = i0 + y;
        if (i >= n || j >= n) continue;
        const double cr = sr[threadIdx.x][y], ci = -si[threadIdx.x][y];
        const size_t o = j + (size_t)i * n;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            double2 p = P[c * NN + o];
            p.x += ph[c].x * cr - ph[c].y * ci;
            p.y += ph[c].x * ci + ph[c].y * cr;
            P[c * NN + o] = p;
        }
    }
}

size_t proj_tc_workspace_floats(int64_t n, int64_t iu) {
    return 6 * (size_t)n * ((iu + 3) / 4 * 4) + 2 * (size_t)n * n + 2 * (size_t)n + 256;
}

// ------------------------------------------------------------------ exact projector
// With FP64-accurate eigenvectors (the eigenpair refinement), C = conj(X) X^T must keep that
// accuracy: the TF32 hi/lo product above leaves ~1e-7 |C|.  The exact variant cuts every row of
// X_k into PROJ_SLICES integer slices (x = 2^e_i sum_s x_s 2^-(8 + 9 s), |x_s| <= 256, e_i the
// row's power-of-two scale), sums the slice products with s + t <= PROJ_DEPTH in the exact-block
// mode of the tcgen05 GEMM (integer blocks of 256, double-float accumulation) and stores C in
// FP64: about 2^-52 of max |x|^2 per term.
constexpr int PROJ_SLICES = 4, PROJ_DEPTH = 3;

// per-row power-of-two scale of X (n x K, column-major): expo[i] = max_k exponent of |X_ik|
__global__ void k_proj_row_expo(const double2* __restrict__ X, int64_t ldx, int64_t n, int64_t K,
                                int* __restrict__ expo) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double m = 0.0;
    for (int64_t k = blockIdx.y; k < K; k += gridDim.y) {
        const double2 x = X[i + k * ldx];
        m = fmax(m, fmax(fabs(x.x), fabs(x.y)));
    }
    int e = -1074;
    if (m > 0.0) frexp(m, &e);   // m < 2^e
    atomicMax(expo + i, e);
}

// X -> 3 S planes with band-contiguous K (Re slices 0..S-1, Im S..2S-1, -Im 2S..3S-1), element
// (i, k) at i * ldk + k; plus the FP64 diagonal sum_k |X_ik|^2 into diag[i].
__global__ void k_stage_proj_exact(const double2* __restrict__ X, int64_t ldx, int64_t n, int64_t K, int64_t ldk,
                                   const int* __restrict__ expo, float* __restrict__ Xt, double* __restrict__ diag) {
    __shared__ double2 tile[32][33];
    __shared__ double dpart[8][32];
    const int64_t i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    double dsum = 0.0;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int64_t i = i0 + threadIdx.x, k = k0 + q;
        const double2 x = (i < n && k < K) ? X[i + k * ldx] : make_double2(0.0, 0.0);
        tile[q][threadIdx.x] = x;
        dsum += x.x * x.x + x.y * x.y;
    }
    dpart[threadIdx.y][threadIdx.x] = dsum;
    __syncthreads();
    if (threadIdx.y == 0 && i0 + threadIdx.x < n) {
        double t = 0.0;
        for (int y = 0; y < (int)blockDim.y; ++y) t += dpart[y][threadIdx.x];
        atomicAdd(diag + i0 + threadIdx.x, t);
    }
    const size_t P = (size_t)n * ldk;
    constexpr int S = PROJ_SLICES;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int64_t i = i0 + q, k = k0 + threadIdx.x;
        if (i < n && k < ldk) {
            const double2 x = tile[threadIdx.x][q];
            const int e = expo[i];
            double a[2] = {ldexp(x.x, -e), ldexp(x.y, -e)};   // |a| < 1, exact
            const size_t o = (size_t)i * ldk + k;
            for (int part = 0; part < 2; ++part) {
                double t = a[part] * 256.0;
                for (int r = 0; r < S; ++r) {
                    const double v = rint(t);                   // |v| <= 256
                    t = (t - v) * 512.0;
                    Xt[(part * S + r) * P + o] = (float)v;
                    if (part == 1) Xt[(2 * S + r) * P + o] = (float)(-v);
                }
            }
        }
    }
}

// exact-block epilogue: the lower triangle of Re C or Im C in FP64, scaled back by 2^(e_i + e_j)
struct ProjStoreExactEpi {
    double* C;
    const int* expo;
    int64_t n;
    __device__ void operator()(int64_t, int64_t row, int64_t col0, const double* v, int64_t M, int64_t N) const {
        if (row >= M) return;
        const int er = expo[row];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
            const int64_t j = col0 + q;
            if (j < N && j <= row) C[row + j * n] = ldexp(v[q], er + expo[j]);
        }
    }
};

size_t proj_tc_exact_workspace_bytes(int64_t n, int64_t iu) {
    const size_t ldk = (size_t)((iu + 3) / 4 * 4);
    return 3 * PROJ_SLICES * (size_t)n * ldk * 4 + 2 * (size_t)n * n * 8 + (size_t)n * 8 + (size_t)n * 4 + 4 * 256;
}

// P_c += ph_c * conj(X) X^T over the first K columns of X, FP64-accurate (exact sliced products).
int bulk_projector_tc_exact(cudaStream_t st, const double2* X, int64_t ldx, int64_t n, int64_t K, int64_t iu,
                            const double2 ph[4], double2* P, void* ws, int* err) {
    if (K <= 0) return 0;
    const int64_t ldk = (iu + 3) / 4 * 4;
    constexpr int S = PROJ_SLICES;
    prof_begin(ST_PROJECTOR);
    auto al = [](char* p) { return (char*)(((uintptr_t)p + 255) & ~(uintptr_t)255); };
    char* p = al(static_cast<char*>(ws));
    float* Xt = (float*)p;
    double* Cr = (double*)al(p + 3 * S * (size_t)n * ldk * 4);
    double* Ci = Cr + (size_t)n * n;
    double* diag = (double*)al((char*)(Ci + (size_t)n * n));
    int* expo = (int*)al((char*)(diag + n));
    FORGE_CUDA(cudaMemsetAsync(diag, 0, n * sizeof(double), st));
    // every row's atomicMax raises its entry from 0x80808080 (far below any exponent) to >= -1074
    FORGE_CUDA(cudaMemsetAsync(expo, 0x80, n * sizeof(int), st));
    k_proj_row_expo<<<dim3((unsigned)((n + 255) / 256), 16), 256, 0, st>>>(X, ldx, n, K, expo);
    FORGE_LAUNCH_CHECK();
    k_stage_proj_exact<<<dim3((unsigned)((n + 31) / 32), (unsigned)((K + 31) / 32)), dim3(32, 8), 0, st>>>(
        X, ldx, n, K, ldk, expo, Xt, diag);
    FORGE_LAUNCH_CHECK();
    std::vector<std::pair<int, int>> pairs;
    for (int d = 0; d <= PROJ_DEPTH; ++d)
        for (int a = 0; a <= d; ++a) pairs.push_back({a, d - a});
    const int nseg = 2 * (int)pairs.size();
    const int32_t nkp = (int32_t)((K + 255) / 256 * 8);
    auto maps = [&](int part, TcKMap& ka, TcKMap& kb) {
        ka = TcKMap{};
        kb = TcKMap{};
        ka.nkp = kb.nkp = nkp;
        ka.nseg = kb.nseg = nseg;
        int q = 0;
        for (auto [a, b] : pairs) {
            const int8_t sc = (int8_t)(16 + 9 * (a + b));
            // Re C = Xr Xr^T + Xi Xi^T; Im C = Xr Xi^T - Xi Xr^T (A = conj(X) rows, B = X rows)
            ka.zsel[q] = a;
            kb.zsel[q] = part == 0 ? b : S + b;
            ka.sexp[q++] = sc;
            ka.zsel[q] = part == 0 ? S + a : 2 * S + a;
            kb.zsel[q] = part == 0 ? S + b : b;
            ka.sexp[q++] = sc;
        }
    };
    TcOperand op{Xt, n, K, ldk, n * ldk, 3 * S};
    for (int part = 0; part < 2; ++part) {
        TcKMap ka, kb;
        maps(part, ka, kb);
        FORGE_TRY((tc_gemm_tf32_mapped<ProjStoreExactEpi, 8, true>(st, op, ka, op, kb, 1, 1,
                                                                    ProjStoreExactEpi{part ? Ci : Cr, expo, n}, err)));
    }
    const unsigned nt = (unsigned)((n + 31) / 32);
    k_proj_accum<double><<<dim3(nt, nt), dim3(32, 8), 0, st>>>(P, Cr, Ci, diag, n, ph[0], ph[1], ph[2], ph[3]);
    FORGE_LAUNCH_CHECK();
    const double nd = (double)n;
    prof_end(ST_PROJECTOR, nd * K * 16.0 + 2.0 * 4.0 * 2.0 * nd * nd * 16.0,
             2.0 * 2.0 * nd * nd * (double)nseg * K / 2.0);
    return 0;
}

// P_c += ph_c * conj(X) X^T over the first K columns of X (n x K, ldx) on the tensor cores.
int bulk_projector_tc(cudaStream_t st, const double2* X, int64_t ldx, int64_t n, int64_t K, int64_t iu,
                      const double2 ph[4], double2* P, float* ws, int* err) {
    if (K <= 0) return 0;
    const int64_t ldk = (iu + 3) / 4 * 4;
    prof_begin(ST_PROJECTOR);
    float* Cr = ws + 6 * (size_t)n * ldk;
    Cr = (float*)(((uintptr_t)Cr + 255) & ~(uintptr_t)255);
    float* Ci = Cr + (size_t)n * n;
    double* diag = (double*)(((uintptr_t)(Ci + (size_t)n * n) + 255) & ~(uintptr_t)255);
    FORGE_CUDA(cudaMemsetAsync(diag, 0, n * sizeof(double), st));
    dim3 g((unsigned)((n + 31) / 32), (unsigned)((K + 31) / 32));
    k_stage_proj<<<g, dim3(32, 8), 0, st>>>(X, ldx, n, K, ldk, ws, diag);
    FORGE_LAUNCH_CHECK();
    const int64_t nkp = (K + 31) / 32;
    TcOperand op{ws, n, K, ldk, n * ldk, 6};
    auto mk = [&](const int32_t* zs) {
        TcKMap m{};
        m.nkp = (int32_t)nkp;
        m.nseg = 6;
        m.koff = 0;
        m.zbatch = 0;
        for (int q = 0; q < 6; ++q) m.zsel[q] = zs[q];
        return m;
    };
    const int32_t za[6] = {0, 1, 0, 1, 2, 3};     // A: hi.re hi.im hi.re hi.im lo.re lo.im
    const int32_t zbr[6] = {0, 1, 2, 3, 0, 1};    // B for Re C: hi.re hi.im lo.re lo.im hi.re hi.im
    const int32_t zbi[6] = {1, 4, 3, 5, 1, 4};    // B for Im C: hi.im -hi.re lo.im -lo.re hi.im -hi.re
    FORGE_TRY(tc_gemm_tf32_mapped(st, op, mk(za), op, mk(zbr), 1, 1, ProjStoreEpi{Cr, n}, err));
    FORGE_TRY(tc_gemm_tf32_mapped(st, op, mk(za), op, mk(zbi), 1, 1, ProjStoreEpi{Ci, n}, err));
    const unsigned nt = (unsigned)((n + 31) / 32);
    k_proj_accum<float><<<dim3(nt, nt), dim3(32, 8), 0, st>>>(P, Cr, Ci, diag, n, ph[0], ph[1], ph[2], ph[3]);
    FORGE_LAUNCH_CHECK();
    const double nd = (double)n;
    prof_end(ST_PROJECTOR, nd * K * 16.0 + 2.0 * 4.0 * 2.0 * nd * nd * 16.0, 2.0 * 2.0 * nd * nd * 6.0 * K / 2.0);
    return 0;
}

}  // namespace forge
