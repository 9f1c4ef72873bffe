// K5 on the tensor cores: C_k = conj(X) X^T over the occupied columns of X_k, accumulated with
// the integer Bloch phases into the four FP64 cells of P(R) (Solve, HartreeFock.f90:456-473).
//
// X_k is split into TF32 planes with orbital rows and band-contiguous K:
//   0 hi.re  1 hi.im  2 lo.re  3 lo.im  4 -hi.re  5 -lo.re
// Re C = Xr Xr^T + Xi Xi^T and Im C = Xr Xi^T - Xi Xr^T are two real GEMMs whose K runs over six
// plane segments (hi*hi + hi*lo + lo*hi for each product), so no operand is copied or negated
// per GEMM.  Only lower tiles are formed; the epilogue writes (i, j) and (j, i).
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
__global__ void __launch_bounds__(256) k_proj_accum(double2* __restrict__ P, const float* __restrict__ Cr,
                                                    const float* __restrict__ Ci, const double* __restrict__ diag,
                                                    int64_t n, double2 ph0, double2 ph1, double2 ph2, double2 ph3) {
    const int64_t bi = blockIdx.x, bj = blockIdx.y;
    if (bi < bj) return;
    __shared__ float sr[32][33], si[32][33];
    const int64_t i0 = bi * 32, j0 = bj * 32;
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int64_t i = i0 + threadIdx.x, j = j0 + y;
        const bool ok = i < n && j < n && i >= j;
        sr[y][threadIdx.x] = ok ? Cr[i + j * n] : 0.f;                 // sr[col][row]
        si[y][threadIdx.x] = (ok && i != j) ? Ci[i + j * n] : 0.f;
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
    k_proj_accum<<<dim3(nt, nt), dim3(32, 8), 0, st>>>(P, Cr, Ci, diag, n, ph[0], ph[1], ph[2], ph[3]);
    FORGE_LAUNCH_CHECK();
    const double nd = (double)n;
    prof_end(ST_PROJECTOR, nd * K * 16.0 + 2.0 * 4.0 * 2.0 * nd * nd * 16.0, 2.0 * 2.0 * nd * nd * 6.0 * K / 2.0);
    return 0;
}

}  // namespace forge
