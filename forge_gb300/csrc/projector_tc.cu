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

// X (n x K columns of X_k, column-major, FP64) -> 6 planes (n rows x ldk, band contiguous)
__global__ void k_stage_proj(const double2* __restrict__ X, int64_t ldx, int64_t n, int64_t K, int64_t ldk,
                             float* __restrict__ Xt) {
    __shared__ double2 tile[32][33];
    const int64_t i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        const int64_t i = i0 + threadIdx.x, k = k0 + q;
        tile[q][threadIdx.x] = (i < n && k < K) ? X[i + k * ldx] : make_double2(0.0, 0.0);
    }
    __syncthreads();
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

struct ProjTcEpi {
    double2* P;     // 4 x n x n
    int64_t n;
    double2 ph[4];
    int imag;       // 0: v = Re C, 1: v = Im C
    __device__ void operator()(int64_t b, int64_t row, int64_t col0, const float* v, int64_t M, int64_t N) const {
        (void)b;
        const int64_t i = row;
        if (i >= M) return;
        const size_t NN = (size_t)n * n;
#pragma unroll 4
        for (int q = 0; q < 32; ++q) {
            const int64_t j = col0 + q;
            if (j >= N || j > i || (imag && j == i)) continue;
            const double c = (double)v[q];
            const size_t oij = i + (size_t)j * n, oji = j + (size_t)i * n;
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) {
                const double2 p = ph[cc];
                double2 a, t;
                if (!imag) {
                    a = make_double2(p.x * c, p.y * c);       // ph * Re C
                    t = a;                                    // (j,i): ph * conj(C) has the same real part
                } else {
                    a = make_double2(-p.y * c, p.x * c);      // ph * (i Im C)
                    t = make_double2(p.y * c, -p.x * c);      // ph * (-i Im C)
                }
                double2* x = P + cc * NN + oij;
                *x = make_double2(x->x + a.x, x->y + a.y);
                if (i != j) {
                    double2* y = P + cc * NN + oji;
                    *y = make_double2(y->x + t.x, y->y + t.y);
                }
            }
        }
    }
};

size_t proj_tc_workspace_floats(int64_t n, int64_t iu) { return 6 * (size_t)n * ((iu + 3) / 4 * 4) + 64; }

// P_c += ph_c * conj(X) X^T over the first K columns of X (n x K, ldx) on the tensor cores.
int bulk_projector_tc(cudaStream_t st, const double2* X, int64_t ldx, int64_t n, int64_t K, int64_t iu,
                      const double2 ph[4], double2* P, float* ws, int* err) {
    if (K <= 0) return 0;
    const int64_t ldk = (iu + 3) / 4 * 4;
    prof_begin(ST_PROJECTOR);
    dim3 g((unsigned)((n + 31) / 32), (unsigned)((K + 31) / 32));
    k_stage_proj<<<g, dim3(32, 8), 0, st>>>(X, ldx, n, K, ldk, ws);
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
    ProjTcEpi er{P, n, {ph[0], ph[1], ph[2], ph[3]}, 0};
    ProjTcEpi ei{P, n, {ph[0], ph[1], ph[2], ph[3]}, 1};
    FORGE_TRY(tc_gemm_tf32_mapped(st, op, mk(za), op, mk(zbr), 1, 1, er, err));
    FORGE_TRY(tc_gemm_tf32_mapped(st, op, mk(za), op, mk(zbi), 1, 1, ei, err));
    const double nd = (double)n;
    prof_end(ST_PROJECTOR, nd * K * 16.0 + 2.0 * 4.0 * 2.0 * nd * nd * 16.0, 2.0 * 2.0 * nd * nd * 6.0 * K / 2.0);
    return 0;
}

}  // namespace forge
