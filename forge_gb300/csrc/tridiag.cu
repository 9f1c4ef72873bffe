// Batched Householder tridiagonalisation (see tridiag.cuh for the structure).
//
// Bytes per column step (algorithmic): the trailing lower triangle, (n-col)^2/2
// complex elements, read once by trd_hemv; the rank-2k update is GEMM-shaped.
#include "tridiag.cuh"
#include "zgemm_engine.cuh"

namespace forge {

namespace {

template <class V>
__device__ inline V ldv(const V* p) {
    return *p;
}

// Block-wide sum (blockDim.x == 256) in the working precision T: the FP32 path keeps its
// per-element arithmetic off the FP64 pipe, which runs at 1/64 of the FP32 rate on this GPU.
template <class T>
__device__ inline T warp_sum_t(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
template <class T>
__device__ inline T block_sum_256(T v, T* sh) {
    v = warp_sum_t(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = v;
    __syncthreads();
    T r = (T)0;
    if (threadIdx.x < 32) {
        r = (l < 8) ? sh[l] : (T)0;
        r = warp_sum_t(r);
    }
    __syncthreads();
    return r;  // valid in thread 0
}

// "last CTA" detection for a per-batch counter; returns true in every thread of the last CTA.
__device__ inline bool last_cta(unsigned* counter, unsigned total) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = atomicAdd(counter, 1u);
        is_last = (t == total - 1);
        if (is_last) *counter = 0u;
    }
    __syncthreads();
    return is_last;
}

}  // namespace

// ---------------------------------------------------------------- trd_col (zlatrd column update + zlarfg)
template <class T>
__global__ void __launch_bounds__(TRD_ROWS) k_trd_col(TrdArgs<T> a, int64_t p, int ii, int64_t col, int has_refl) {
    using V = typename CV<T>::type;
    const int64_t b = blockIdx.y, n = a.n, lda = a.lda;
    V* A = a.A + b * a.strideA;
    V* W = a.W + b * (n * TRD_NB);
    __shared__ V wrow[TRD_NB], arow[TRD_NB];
    __shared__ T sh[8];
    if (threadIdx.x < ii) {
        wrow[threadIdx.x] = W[col + threadIdx.x * n];
        arow[threadIdx.x] = A[col + (p + threadIdx.x) * lda];
    }
    __syncthreads();
    const int64_t r = col + (int64_t)blockIdx.x * TRD_ROWS + threadIdx.x;
    T nrm = (T)0;
    if (r < n) {
        V x = A[r + col * lda];
        for (int l = 0; l < ii; ++l) {
            x = vsub(x, vmulcj(A[r + (p + l) * lda], wrow[l]));
            x = vsub(x, vmulcj(W[r + l * n], arow[l]));
        }
        if (r == col) {
            x.y = 0;
            a.d[b * n + col] = (double)x.x;
        }
        A[r + col * lda] = x;
        double* sc = a.scal + b * 16;
        if (r == col + 1) {
            sc[0] = (double)x.x;
            sc[1] = (double)x.y;
        }
        if (r >= col + 2) nrm = x.x * x.x + x.y * x.y;
    }
    const T s = block_sum_256(nrm, sh);
    double* part = a.part + b * a.pstride;
    if (threadIdx.x == 0) part[blockIdx.x] = (double)s;
    if (last_cta(a.cnt + b * 4, gridDim.x) && threadIdx.x == 0) {
        double xn2 = 0.0;
        for (unsigned q = 0; q < gridDim.x; ++q) xn2 += ((volatile double*)part)[q];
        double* sc = a.scal + b * 16;
        V* tau = a.tau + b * n;
        if (!has_refl) {
            tau[col] = vzero<V>();
            sc[2] = 1.0;
            sc[3] = 0.0;
            sc[4] = 0.0;
            sc[5] = 0.0;
            return;
        }
        const double ar = ((volatile double*)sc)[0], ai = ((volatile double*)sc)[1];
        // zlarfg: beta = -sign(|(alpha, x)|, Re alpha), tau = (beta - alpha)/beta, x *= 1/(alpha - beta)
        if (xn2 == 0.0 && ai == 0.0) {
            tau[col] = vzero<V>();
            sc[2] = 1.0;
            sc[3] = 0.0;
            sc[4] = 0.0;
            sc[5] = 0.0;
            a.e[b * n + col] = ar;
        } else {
            double beta = -copysign(sqrt(ar * ar + ai * ai + xn2), ar);
            double tr = (beta - ar) / beta, ti = -ai / beta;
            // 1/(alpha - beta)
            double dr = ar - beta, di = ai;
            double den = dr * dr + di * di;
            sc[2] = dr / den;
            sc[3] = -di / den;
            sc[4] = tr;
            sc[5] = ti;
            tau[col] = vmake<V>((T)tr, (T)ti);
            a.e[b * n + col] = beta;
        }
    }
}

// ---------------------------------------------------------------- trd_hemv (+ panel dots)
template <class T>
__device__ inline typename CV<T>::type trd_v(const typename CV<T>::type* A, int64_t lda, int64_t col, int64_t r,
                                             double sr, double si) {
    using V = typename CV<T>::type;
    if (r == col + 1) return vmake<V>((T)1, (T)0);
    const V x = A[r + col * lda];
    const T tr = (T)sr, ti = (T)si;
    return vmake<V>(x.x * tr - x.y * ti, x.x * ti + x.y * tr);
}

template <class T>
__global__ void __launch_bounds__(256) k_trd_hemv(TrdArgs<T> a, int64_t p, int ii, int64_t col, int64_t ntiles) {
    using V = typename CV<T>::type;
    const int64_t b = blockIdx.y, n = a.n, lda = a.lda;
    const V* A = a.A + b * a.strideA;
    const double* sc = a.scal + b * 16;
    const double sr = sc[2], si = sc[3];
    const int64_t c0 = col + 1;
    const int64_t t = blockIdx.x;
    if (t < ntiles) {
        // tile (bi, bj), bj <= bi, of the trailing matrix A(c0:n, c0:n): rows [64 bi, 64 bi + 64),
        // columns [64 bj, 64 bj + 64); t = bi (bi + 1) / 2 + bj
        int64_t bi = (int64_t)((sqrtf(8.f * (float)t + 1.f) - 1.f) * 0.5f);   // corrected below
        while ((bi + 1) * (bi + 2) / 2 <= t) ++bi;
        while (bi * (bi + 1) / 2 > t) --bi;
        const int64_t bj = t - bi * (bi + 1) / 2;
        const int64_t R0 = c0 + bi * HV_RB, C0 = c0 + bj * HV_CB;
        __shared__ V vr[HV_RB], vc[HV_CB];
        __shared__ V rsum[4][HV_RB];
        __shared__ V cs[HV_RB][HV_CB + 1];
        __shared__ V cq[4][HV_CB];
        if (threadIdx.x < HV_RB) {
            const int64_t r = R0 + threadIdx.x;
            vr[threadIdx.x] = (r < n) ? trd_v<T>(A, lda, col, r, sr, si) : vzero<V>();
        } else if (threadIdx.x < HV_RB + HV_CB) {
            const int64_t c = C0 + threadIdx.x - HV_RB;
            vc[threadIdx.x - HV_RB] = (c < n) ? trd_v<T>(A, lda, col, c, sr, si) : vzero<V>();
        }
        const int tr = threadIdx.x & 63, tg = threadIdx.x >> 6;
        const int64_t r0 = R0 + tr;
        // 16 loads per thread (row r0, 16 columns) issued before any arithmetic
        V a0[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int64_t c = C0 + tg * 16 + q;
            a0[q] = (r0 < n && c < n && c <= r0) ? A[r0 + c * lda] : vzero<V>();
        }
        __syncthreads();
        V racc = vzero<V>();
        const V v0 = vr[tr];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int64_t c = C0 + tg * 16 + q;
            V x0 = a0[q];
            const bool d0 = (c == r0);
            if (d0) x0.y = 0;
            racc = vadd(racc, vmul(x0, vc[tg * 16 + q]));
            // column part: conj(A(r, c)) v_r for r > c (the diagonal belongs to the row part only)
            cs[tr][tg * 16 + q] = d0 ? vzero<V>() : vcjmul(x0, v0);
        }
        rsum[tg][tr] = racc;
        __syncthreads();
        {
            // column sums: thread (col, quarter of the 64 rows)
            const int c = threadIdx.x & 63, qt = threadIdx.x >> 6;
            V acc = vzero<V>();
#pragma unroll
            for (int i = 0; i < 16; ++i) acc = vadd(acc, cs[qt * 16 + i][c]);
            cq[qt][c] = acc;
        }
        __syncthreads();
        V* Yrow = a.Yrow + b * a.ystride;
        V* Ycol = a.Ycol + b * a.ystride;
        if (threadIdx.x < HV_RB) {
            const int64_t r = R0 + threadIdx.x;
            if (r < n)
                Yrow[bj * n + r] = vadd(vadd(rsum[0][threadIdx.x], rsum[1][threadIdx.x]),
                                        vadd(rsum[2][threadIdx.x], rsum[3][threadIdx.x]));
        } else if (threadIdx.x < HV_RB + HV_CB) {
            const int q = threadIdx.x - HV_RB;
            const int64_t c = C0 + q;
            if (c < n) Ycol[bi * n + c] = vadd(vadd(cq[0][q], cq[1][q]), vadd(cq[2][q], cq[3][q]));
        }
    } else {
        // panel dots over rows [c0 + rb*256, ...): s1 = W^H v, s2 = V^H v
        const int64_t rb = t - ntiles;
        const int64_t r = c0 + rb * 256 + threadIdx.x;
        const V* W = a.W + b * (n * TRD_NB);
        __shared__ V s1w[8][TRD_NB], s2w[8][TRD_NB];
        V v = (r < n) ? trd_v<T>(A, lda, col, r, sr, si) : vzero<V>();
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int l = 0; l < ii; ++l) {
            V x1 = vzero<V>(), x2 = vzero<V>();
            if (r < n) {
                x1 = vcjmul(W[r + l * n], v);
                x2 = vcjmul(A[r + (p + l) * lda], v);
            }
            x1 = warp_sum(x1);
            x2 = warp_sum(x2);
            if (lane == 0) {
                s1w[w][l] = x1;
                s2w[w][l] = x2;
            }
        }
        __syncthreads();
        V* S = a.Spart + b * a.sstride + rb * 2 * TRD_NB;
        if (threadIdx.x < ii) {
            V x1 = vzero<V>(), x2 = vzero<V>();
            for (int q = 0; q < 8; ++q) {
                x1 = vadd(x1, s1w[q][threadIdx.x]);
                x2 = vadd(x2, s2w[q][threadIdx.x]);
            }
            S[threadIdx.x] = x1;
            S[TRD_NB + threadIdx.x] = x2;
        }
    }
}

// ---------------------------------------------------------------- trd_finish
template <class T>
__global__ void __launch_bounds__(TRD_ROWS) k_trd_finish(TrdArgs<T> a, int64_t p, int ii, int64_t col, int64_t nb2,
                                                         int64_t nrb) {
    using V = typename CV<T>::type;
    const int64_t b = blockIdx.y, n = a.n, lda = a.lda;
    V* A = a.A + b * a.strideA;
    V* W = a.W + b * (n * TRD_NB);
    double* sc = a.scal + b * 16;
    const double sr = sc[2], si = sc[3];
    const V tau = vmake<V>((T)sc[4], (T)sc[5]);
    const int64_t c0 = col + 1;
    __shared__ V s1[TRD_NB], s2[TRD_NB];
    __shared__ T sh[8];
    if (threadIdx.x < ii) {
        const V* S = a.Spart + b * a.sstride;
        V x1 = vzero<V>(), x2 = vzero<V>();
        for (int64_t q = 0; q < nrb; ++q) {
            x1 = vadd(x1, S[q * 2 * TRD_NB + threadIdx.x]);
            x2 = vadd(x2, S[q * 2 * TRD_NB + TRD_NB + threadIdx.x]);
        }
        s1[threadIdx.x] = x1;
        s2[threadIdx.x] = x2;
    }
    // 32 rows per CTA, 8 threads per row share the sum over the Yrow / Ycol partial slots
    __shared__ V ysl[8][33];
    const int rr = threadIdx.x & 31, sl = threadIdx.x >> 5;
    const int64_t r = c0 + (int64_t)blockIdx.x * 32 + rr;
    if (r < n) {
        // row part from the tiles (blk128(r), bj <= blk64(r)); column part from (bi >= blk128(r), blk64(r))
        const int64_t Bc = (r - c0) / HV_CB, Br = (r - c0) / HV_RB;
        const V* Yrow = a.Yrow + b * a.ystride;
        const V* Ycol = a.Ycol + b * a.ystride;
        V y = vzero<V>();
        for (int64_t q = sl; q <= Bc; q += 8) y = vadd(y, Yrow[q * n + r]);
        for (int64_t q = Br + sl; q < nb2; q += 8) y = vadd(y, Ycol[q * n + r]);
        ysl[sl][rr] = y;
    }
    __syncthreads();   // s1, s2 and the slot sums are in shared memory
    if (r < n) {
        // the panel corrections -V s1 - W s2, split over the 8 slices
        V y = ysl[sl][rr];
        for (int l = sl; l < ii; l += 8) {
            y = vsub(y, vmul(A[r + (p + l) * lda], s1[l]));
            y = vsub(y, vmul(W[r + l * n], s2[l]));
        }
        ysl[sl][rr] = y;
    }
    __syncthreads();
    T dre = (T)0, dim = (T)0;
    if (sl == 0 && r < n) {
        V y = vzero<V>();
#pragma unroll
        for (int q = 0; q < 8; ++q) y = vadd(y, ysl[q][rr]);
        y = vmul(tau, y);
        V v = trd_v<T>(A, lda, col, r, sr, si);
        A[r + col * lda] = v;
        W[r + ii * n] = y;
        // zdotc(w, v) = sum conj(w) v
        V cv = vcjmul(y, v);
        dre = cv.x;
        dim = cv.y;
    }
    const T s_re = block_sum_256(dre, sh);
    const T s_im = block_sum_256(dim, sh);
    double* part = a.part + b * a.pstride;
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = (double)s_re;
        part[2 * blockIdx.x + 1] = (double)s_im;
    }
    if (last_cta(a.cnt + b * 4 + 1, gridDim.x) && threadIdx.x == 0) {
        double xr = 0.0, xi = 0.0;
        for (unsigned q = 0; q < gridDim.x; ++q) {
            xr += ((volatile double*)part)[2 * q];
            xi += ((volatile double*)part)[2 * q + 1];
        }
        // alpha2 = -1/2 tau (w^H v)
        const double tr = sc[4], ti = sc[5];
        sc[6] = -0.5 * (tr * xr - ti * xi);
        sc[7] = -0.5 * (tr * xi + ti * xr);
    }
}

template <class T>
__global__ void __launch_bounds__(TRD_ROWS) k_trd_fix(TrdArgs<T> a, int ii, int64_t col) {
    using V = typename CV<T>::type;
    const int64_t b = blockIdx.y, n = a.n, lda = a.lda;
    const V* A = a.A + b * a.strideA;
    V* W = a.W + b * (n * TRD_NB);
    const double* sc = a.scal + b * 16;
    const V al = vmake<V>((T)sc[6], (T)sc[7]);
    const int64_t r = col + 1 + (int64_t)blockIdx.x * TRD_ROWS + threadIdx.x;
    if (r < n) W[r + ii * n] = vadd(W[r + ii * n], vmul(al, A[r + col * lda]));
}

// ---------------------------------------------------------------- rank-2k trailing update
template <class V>
struct Her2kA {
    const V* A;
    const V* W;
    int64_t lda, strideA, n, strideW, r0, p, w;
    __device__ V operator()(int64_t i, int64_t k) const {
        const int64_t r = r0 + i, b = blockIdx.z;
        if (r >= n || k >= 2 * w) return vzero<V>();
        if (k < w) return A[b * strideA + r + (p + k) * lda];
        return W[b * strideW + r + (k - w) * n];
    }
};
template <class V>
struct Her2kB {
    const V* A;
    const V* W;
    int64_t lda, strideA, n, strideW, r0, p, w;
    __device__ V operator()(int64_t j, int64_t k) const {
        const int64_t r = r0 + j, b = blockIdx.z;
        if (r >= n || k >= 2 * w) return vzero<V>();
        if (k < w) return vconj(W[b * strideW + r + k * n]);
        return vconj(A[b * strideA + r + (p + k - w) * lda]);
    }
};
template <class V>
struct Her2kEpi {
    V* A;
    int64_t lda, strideA, r0;
    __device__ void operator()(int64_t i, int64_t j, V c) const {
        V* x = A + blockIdx.z * strideA + (r0 + i) + (r0 + j) * lda;
        V y = vsub(*x, c);
        if (i == j) y.y = 0;
        *x = y;
    }
};

template <class T>
int her2k_update(cudaStream_t st, TrdArgs<T>& a, int64_t p, int64_t w, int64_t batch) {
    using V = typename CV<T>::type;
    const int64_t r0 = p + w, m = a.n - r0;
    if (m <= 0) return 0;
    Her2kA<V> fa{a.A, a.W, a.lda, a.strideA, a.n, a.n * TRD_NB, r0, p, w};
    Her2kB<V> fb{a.A, a.W, a.lda, a.strideA, a.n, a.n * TRD_NB, r0, p, w};
    Her2kEpi<V> ep{a.A, a.lda, a.strideA, r0};
    return zgemm_launch<V, IMAJOR, IMAJOR, true>(st, m, m, 2 * w, batch, fa, fb, ep);
}

// ---------------------------------------------------------------- driver
template <class T>
int tridiagonalize(cudaStream_t st, TrdArgs<T>& a, int64_t batch) {
    const int64_t n = a.n;
    for (int64_t p = 0; p < n; p += TRD_NB) {
        const int64_t w = (n - p < TRD_NB) ? (n - p) : TRD_NB;
        int64_t nrefl = 0;
        for (int ii = 0; ii < w; ++ii) {
            const int64_t col = p + ii;
            const int has_refl = (col < n - 1) ? 1 : 0;
            const double esz = (double)sizeof(typename CV<T>::type);
            dim3 ga((unsigned)((n - col + TRD_ROWS - 1) / TRD_ROWS), (unsigned)batch);
            prof_begin(ST_TRD_COL);
            k_trd_col<T><<<ga, TRD_ROWS, 0, st>>>(a, p, ii, col, has_refl);
            FORGE_LAUNCH_CHECK();
            prof_end(ST_TRD_COL, batch * (double)(n - col) * (2.0 * ii + 2.0) * esz, 0.0);
            if (!has_refl) continue;
            ++nrefl;
            const int64_t n2 = n - col - 1;
            const int64_t nbr = (n2 + HV_RB - 1) / HV_RB;   // 64-row blocks (= 64-column blocks)
            const int64_t ntiles = nbr * (nbr + 1) / 2;     // row block bi holds bi + 1 tiles
            const int64_t nrb = (n2 + 255) / 256;
            dim3 gb((unsigned)(ntiles + (ii > 0 ? nrb : 0)), (unsigned)batch);
            prof_begin(ST_HEMV);
            k_trd_hemv<T><<<gb, 256, 0, st>>>(a, p, ii, col, ntiles);
            FORGE_LAUNCH_CHECK();
            // algorithmic traffic: the trailing lower triangle read once
            prof_end(ST_HEMV, batch * 0.5 * (double)n2 * (double)(n2 + 1) * esz, batch * 8.0 * (double)n2 * n2);
            dim3 gf((unsigned)((n2 + 31) / 32), (unsigned)batch);
            dim3 gc((unsigned)((n2 + TRD_ROWS - 1) / TRD_ROWS), (unsigned)batch);
            prof_begin(ST_TRD_FINISH);
            k_trd_finish<T><<<gf, TRD_ROWS, 0, st>>>(a, p, ii, col, nbr, ii > 0 ? nrb : 0);
            FORGE_LAUNCH_CHECK();
            k_trd_fix<T><<<gc, TRD_ROWS, 0, st>>>(a, ii, col);
            FORGE_LAUNCH_CHECK();
            prof_end(ST_TRD_FINISH, batch * (double)n2 * (2.0 * ii + 4.0) * esz, 0.0);
        }
        if (nrefl > 0 && p + w < n) {
            const double m2 = (double)(n - p - w);
            prof_begin(ST_HER2K);
            if (a.her2k)
                FORGE_TRY(a.her2k(st, a, p, nrefl, batch, a.her2k_user));
            else
                FORGE_TRY(her2k_update<T>(st, a, p, nrefl, batch));
            prof_end(ST_HER2K, batch * m2 * m2 * (double)sizeof(typename CV<T>::type),
                     batch * 8.0 * m2 * m2 * (double)nrefl);  // lower half of 2*nrefl complex MACs
        }
    }
    return 0;
}

template int tridiagonalize<double>(cudaStream_t, TrdArgs<double>&, int64_t);
template int tridiagonalize<float>(cudaStream_t, TrdArgs<float>&, int64_t);

}  // namespace forge
