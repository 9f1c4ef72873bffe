// Mixed-precision batched eigen-solver (FORGE_PREC_MIXED).
//
//  1. H(k) (complex128) -> complex64 working copy.
//  2. Householder tridiagonalisation with the FP32 column kernels (hemv on the CUDA cores,
//     HBM-bound) and the trailing rank-2k update A22 -= V W^H + W V^H on the tcgen05 tensor
//     cores: the complex product is one real GEMM with interleaved real/imaginary output rows,
//     each operand split into TF32 hi + lo parts (a*b ~ ah*bh + ah*bl + al*bh, FP32 accuracy),
//     accumulated in FP32 in TMEM.
//  3. Eigenvalues (bisection) and tridiagonal eigenvectors (inverse iteration) in FP64.
//  4. Back-transformation X = Q Z in compact-WY blocks of 64 reflectors: W = V^H X and
//     X -= V (T W) on the tensor cores with the same split; X lives in four TF32 planes
//     (hi.re, hi.im, lo.re, lo.im) that the second GEMM's epilogue re-splits in place.
//  5. X -> complex128 for the projectors.
#include <algorithm>

#include "cvec.cuh"
#include "eig.cuh"
#include "tc_gemm.cuh"
#include "zgemm_engine.cuh"

namespace forge {

constexpr int BT_NB = 64;   // reflectors per back-transform block
constexpr int64_t BT_CTA_TARGET = 2 * 152;  // CTAs that fill the GPU (two resident per SM)

// Upper bounds of the K splits of the two long-K back-transform products (they size the
// workspace): the Gram matrix V^H V (one 64 x 64 tile per matrix, no split shorter than 256
// rows) and W = V^H X on the tensor cores (iu/128 tiles per matrix, >= 8 K blocks per split).
inline void bt_split_caps(int64_t n, int64_t iu, int64_t batch, int64_t& ksg, int64_t& ksw) {
    ksg = std::min<int64_t>(std::min<int64_t>(32, (BT_CTA_TARGET + batch - 1) / batch), (n + 255) / 256);
    const int64_t tiles = (iu + TC_BN - 1) / TC_BN * batch;
    ksw = std::min<int64_t>(std::min<int64_t>(16, (BT_CTA_TARGET + tiles - 1) / tiles),
                            std::max<int64_t>(1, 6 * ((n + 31) / 32) / 8));
    ksg = std::max<int64_t>(1, ksg);
}
constexpr int HK = 384;     // K'' of the split rank-2k update: 3 splits x (re, im) x 2 x TRD_NB

__device__ inline float tf32_hi(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
__device__ inline void split2(float x, float& hi, float& lo) {
    hi = tf32_hi(x);
    lo = x - hi;
}

struct MixedWs {
    int64_t n, iu, B, n4, Kp, nblk, nrb, pstride;
    float2* A32;
    float2 *W, *Yrow, *Ycol, *Spart, *tau;
    double* part;
    double* scal;
    unsigned* cnt;
    float *SA, *SB;       // rank-2k staging
    float* Xs;            // B x 4 planes x (n4 x iu)
    float *A1, *A2, *B2;  // back-transform staging
    float2 *Wb, *W2, *G, *T;
    int* err;
};

namespace {
inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }
struct Carve {
    char* base;
    size_t off = 0;
    template <class T>
    T* take(size_t count) {
        size_t o = off;
        off = al256(off + count * sizeof(T));
        return base ? reinterpret_cast<T*>(base + o) : nullptr;
    }
};
void carve(MixedWs& w, Carve& c) {
    const int64_t n = w.n, iu = w.iu, B = w.B;
    w.n4 = (n + 3) / 4 * 4;
    w.Kp = (n + 31) / 32 * 32;
    w.nblk = (n + TRD_TILE - 1) / TRD_TILE;
    w.nrb = (n + 255) / 256;
    w.pstride = 2 * ((n + 31) / 32) + 2;  // per-CTA partials of trd_col / trd_finish
    w.A32 = c.take<float2>(B * n * n);
    w.W = c.take<float2>(B * n * TRD_NB);
    w.Yrow = c.take<float2>(B * w.nblk * n);
    w.Ycol = c.take<float2>(B * w.nblk * n);
    w.Spart = c.take<float2>(B * w.nrb * 2 * TRD_NB);
    w.tau = c.take<float2>(B * n);
    w.part = c.take<double>(B * w.pstride);
    w.scal = c.take<double>(B * 16);
    w.cnt = c.take<unsigned>(B * 4);
    w.SA = c.take<float>(B * 2 * n * HK);
    w.SB = c.take<float>(B * n * HK);
    w.Xs = c.take<float>(B * 4 * w.n4 * iu);
    w.A1 = c.take<float>(B * 2 * BT_NB * 6 * w.Kp);
    w.A2 = c.take<float>(B * 2 * n * 6 * BT_NB);
    w.B2 = c.take<float>(B * iu * 6 * BT_NB);
    int64_t ksg, ksw;
    bt_split_caps(n, iu, B, ksg, ksw);
    w.Wb = c.take<float2>(ksw * B * BT_NB * iu);
    w.W2 = c.take<float2>(B * BT_NB * iu);
    w.G = c.take<float2>(ksg * B * BT_NB * BT_NB);
    w.T = c.take<float2>(B * BT_NB * BT_NB);
    w.err = c.take<int>(1);
}
}  // namespace

// the TF32 hi / lo eigenvector planes of the last eig_mixed call on this workspace (four planes of
// n4 x iu floats per matrix: hi.re, hi.im, lo.re, lo.im, column-major)
const float* eig_mixed_planes(void* mixed_ws, int64_t n, int64_t iu, int64_t batch, int64_t* n4) {
    MixedWs w{};
    w.n = n;
    w.iu = iu;
    w.B = batch;
    Carve c{static_cast<char*>(mixed_ws)};
    carve(w, c);
    *n4 = w.n4;
    return w.Xs;
}

size_t eig_mixed_workspace_bytes(int64_t n, int64_t iu, int64_t batch) {
    MixedWs w{};
    w.n = n;
    w.iu = iu;
    w.B = batch;
    Carve c{nullptr};
    carve(w, c);
    return c.off;
}

// ---------------------------------------------------------------- conversions
__global__ void k_h_to_f32(const double2* __restrict__ H, float2* __restrict__ A, size_t total) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x)
        A[q] = make_float2((float)H[q].x, (float)H[q].y);
}

// Z (row-major n x iu, FP64) -> planes hi.re, hi.im(=0), lo.re, lo.im(=0), column-major with pitch n4
__global__ void k_z_to_planes(const double* __restrict__ Z, int64_t n, int64_t n4, int64_t iu,
                              float* __restrict__ Xs) {
    const int64_t b = blockIdx.z;
    __shared__ double tile[32][33];
    const int64_t r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        int64_t r = r0 + q, c = c0 + threadIdx.x;
        tile[q][threadIdx.x] = (r < n && c < iu) ? Z[b * n * iu + r * iu + c] : 0.0;
    }
    __syncthreads();
    const size_t P = (size_t)n4 * iu;
    float* X = Xs + b * 4 * P;
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        int64_t c = c0 + q, r = r0 + threadIdx.x;
        if (c < iu && r < n4) {
            float hi, lo;
            split2((float)tile[threadIdx.x][q], hi, lo);
            // the FP64 value carries more than TF32 hi+lo: keep the rounding of the FP32 value
            if (r >= n) hi = lo = 0.f;
            const size_t o = (size_t)c * n4 + r;
            X[o] = hi;
            X[P + o] = 0.f;
            X[2 * P + o] = lo;
            X[3 * P + o] = 0.f;
        }
    }
}

__global__ void k_planes_to_x(const float* __restrict__ Xs, int64_t n, int64_t n4, int64_t iu, int64_t ncols,
                              double2* __restrict__ X, int64_t ldx, int64_t strideX) {
    const int64_t b = blockIdx.y;
    const size_t P = (size_t)n4 * iu;
    const float* S = Xs + b * 4 * P;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < (size_t)n * ncols;
         q += (size_t)gridDim.x * blockDim.x) {
        const int64_t c = q / n, r = q - c * n;
        const size_t o = (size_t)c * n4 + r;
        X[b * strideX + r + c * ldx] =
            make_double2((double)S[o] + (double)S[2 * P + o], (double)S[P + o] + (double)S[3 * P + o]);
    }
}

// Unit 2-norm of every eigenvector column in FP64: the FP32 reflectors leave column norms off
// by O(n eps_32), a systematic error that would otherwise shift the trace of the projectors.
// One CTA (256 threads) per column.
__global__ void __launch_bounds__(256) k_normalize_cols(double2* __restrict__ X, int64_t n, int64_t iu, int64_t ldx,
                                                        int64_t strideX) {
    const int64_t c = blockIdx.x, b = blockIdx.y;
    double2* x = X + b * strideX + c * ldx;
    double s = 0.0;
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) s += x[r].x * x[r].x + x[r].y * x[r].y;
    __shared__ double red[8];
    s = warp_sum_d(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
        t = warp_sum_d(t);
        if (threadIdx.x == 0) red[0] = t;
    }
    __syncthreads();
    const double scl = red[0] > 0.0 ? 1.0 / sqrt(red[0]) : 1.0;
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) x[r] = make_double2(x[r].x * scl, x[r].y * scl);
}

// ---------------------------------------------------------------- rank-2k update on the tensor cores
struct Her2kStageArgs {
    const float2* A;
    const float2* W;
    int64_t lda, strideA, n, r0, p, w;
    float *SA, *SB;
    int64_t saStride, sbStride;
};

// one thread per (row i of the trailing block, l in [0, 2 TRD_NB))
__global__ void k_stage_her2k(Her2kStageArgs s) {
    const int64_t b = blockIdx.y;
    const int64_t m = s.n - s.r0;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t i = t / (2 * TRD_NB);
    const int l = (int)(t - i * 2 * TRD_NB);
    if (i >= m) return;
    const int64_t r = s.r0 + i;
    float2 u = make_float2(0.f, 0.f), z = make_float2(0.f, 0.f);
    const float2* A = s.A + b * s.strideA;
    const float2* W = s.W + b * (s.n * TRD_NB);
    if (l < s.w) {
        u = A[r + (s.p + l) * s.lda];
        z = W[r + l * s.n];
    } else if (l >= TRD_NB && l < TRD_NB + s.w) {
        u = W[r + (l - TRD_NB) * s.n];
        z = A[r + (s.p + l - TRD_NB) * s.lda];
    }
    float urh, url, uih, uil, zrh, zrl, zih, zil;
    split2(u.x, urh, url);
    split2(u.y, uih, uil);
    split2(z.x, zrh, zrl);
    split2(z.y, zih, zil);
    float* ra = s.SA + b * s.saStride + (2 * i) * HK;   // real output row
    float* ia = ra + HK;                                // imaginary output row
    float* rb = s.SB + b * s.sbStride + i * HK;
    // segment g (128 floats): [0,64) multiplies Re Z, [64,128) multiplies Im Z
    ra[l] = urh;        ra[64 + l] = uih;         // hi * hi
    ra[128 + l] = urh;  ra[192 + l] = uih;        // hi * lo
    ra[256 + l] = url;  ra[320 + l] = uil;        // lo * hi
    ia[l] = uih;        ia[64 + l] = -urh;
    ia[128 + l] = uih;  ia[192 + l] = -urh;
    ia[256 + l] = uil;  ia[320 + l] = -url;
    rb[l] = zrh;        rb[64 + l] = zih;
    rb[128 + l] = zrl;  rb[192 + l] = zil;
    rb[256 + l] = zrh;  rb[320 + l] = zih;
}

// epilogue: interleaved rows (2i = Re, 2i+1 = Im) of C = U Z^H; A22(i,j) -= C(i,j) for j <= i.
// The two lanes of a row pair split the 32 columns: the even lane updates columns 0..15, the odd
// lane 16..31, each with 16 independent loads issued before its stores.
struct Her2kTcEpi {
    float2* A;
    int64_t lda, strideA, r0;
    __device__ void operator()(int64_t b, int64_t row, int64_t col0, const float* v, int64_t M, int64_t N) const {
        const int64_t i = row >> 1;
        const bool odd = (row & 1) != 0;
        float other[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) other[q] = __shfl_xor_sync(0xffffffffu, odd ? v[q] : v[16 + q], 1);
        if (row >= M) return;
        const int h0 = odd ? 16 : 0;
        float2* __restrict__ base = A + b * strideA + (r0 + i);
        float2 old[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int64_t j = col0 + h0 + q;
            old[q] = (j < N && j <= i) ? base[(r0 + j) * lda] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int64_t j = col0 + h0 + q;
            if (j < N && j <= i) {
                const float re = odd ? other[q] : v[q];
                const float im = odd ? v[16 + q] : other[q];
                float2 y = old[q];
                y.x -= re;
                y.y = (i == j) ? 0.f : y.y - im;
                base[(r0 + j) * lda] = y;
            }
        }
    }
};

int her2k_tc(cudaStream_t st, TrdArgs<float>& a, int64_t p, int64_t w, int64_t batch, void* user) {
    MixedWs& ws = *static_cast<MixedWs*>(user);
    const int64_t r0 = p + w, m = a.n - r0;
    if (m <= 0) return 0;
    Her2kStageArgs s{a.A, a.W, a.lda, a.strideA, a.n, r0, p, w, ws.SA, ws.SB, 2 * a.n * HK, a.n * HK};
    const int64_t threads = m * 2 * TRD_NB;
    prof_begin(ST_HER2K);
    k_stage_her2k<<<dim3((unsigned)((threads + 255) / 256), (unsigned)batch), 256, 0, st>>>(s);
    FORGE_LAUNCH_CHECK();
    TcOperand A{ws.SA, 2 * m, HK, HK, 2 * a.n * HK};
    TcOperand B{ws.SB, m, HK, HK, a.n * HK};
    FORGE_TRY(tc_gemm_tf32(st, A, B, HK, batch, Her2kTcEpi{a.A, a.lda, a.strideA, r0}, ws.err, 2));
    const double md = (double)m;
    prof_end(ST_HER2K, batch * (md * md * 8.0 + 3.0 * md * HK * 4.0), batch * 2.0 * (2.0 * md) * md * HK / 2.0);
    return 0;
}

// ---------------------------------------------------------------- back-transformation on the tensor cores
__device__ inline float2 bt_v(const float2* A, int64_t lda, int64_t n, int64_t j, int64_t r) {
    // reflector j: v(j+1) = 1, v(r) = A(r, j) for r > j+1, 0 above
    if (r < j + 1 || r >= n) return make_float2(0.f, 0.f);
    if (r == j + 1) return make_float2(1.f, 0.f);
    return A[r + j * lda];
}

struct BtGA {  // a(l, k) = conj(V(j0+1+k, l))   (Gram G = V^H V)
    const float2* A;
    int64_t lda, strideA, n, j0, nbk;
    __device__ float2 operator()(int64_t l, int64_t k) const {
        if (l >= nbk) return make_float2(0.f, 0.f);
        return vconj(bt_v(A + blockIdx.z * strideA, lda, n, j0 + l, j0 + 1 + k));
    }
};
struct BtGB {
    const float2* A;
    int64_t lda, strideA, n, j0, nbk;
    __device__ float2 operator()(int64_t l, int64_t k) const {
        if (l >= nbk) return make_float2(0.f, 0.f);
        return bt_v(A + blockIdx.z * strideA, lda, n, j0 + l, j0 + 1 + k);
    }
};
struct StoreF2 {
    float2* G;
    int64_t ld, stride;
    __device__ void operator()(int64_t i, int64_t j, float2 c) const { G[blockIdx.z * stride + i + j * ld] = c; }
};
// partial Gram of K split s of batch item b at G + (s * batch + b) * BT_NB^2
struct StoreGramSplit {
    float2* G;
    int64_t batch;
    __device__ void operator()(int64_t s, int64_t i, int64_t j, float2 c) const {
        G[(s * batch + blockIdx.z) * BT_NB * BT_NB + i + j * BT_NB] = c;
    }
};
struct TWa {
    const float2* T;
    int64_t nbk;
    __device__ float2 operator()(int64_t l, int64_t q) const {
        if (l >= nbk || q >= nbk || q < l) return make_float2(0.f, 0.f);
        return T[blockIdx.z * BT_NB * BT_NB + l + q * BT_NB];
    }
};
// W(q, c) as the sum of the ks K-split partials of V^H X (partial z = b * ks + s)
struct TWb {
    const float2* W;
    int64_t nbk, iu, ks;
    __device__ float2 operator()(int64_t c, int64_t q) const {
        if (q >= nbk || c >= iu) return make_float2(0.f, 0.f);
        const float2* p = W + (blockIdx.z * ks) * BT_NB * iu + q + c * BT_NB;
        float2 acc = p[0];
        for (int64_t s = 1; s < ks; ++s) acc = vadd(acc, p[s * BT_NB * iu]);
        return acc;
    }
};

// T of the compact-WY form from the Gram matrix G = V^H V, given as ks K-split partials
// (partial s of batch item b at G + (s * batch + b) * BT_NB^2).  blockDim.x = BT_NB.
__global__ void k_larft32(const float2* __restrict__ G, int64_t ks, int64_t batch, const float2* __restrict__ tau,
                          int64_t n, int64_t j0, int64_t nbk, float2* __restrict__ T) {
    const int64_t b = blockIdx.x;
    float2* Tb = T + b * BT_NB * BT_NB;
    const float2* tb = tau + b * n;
    __shared__ float2 tmp[BT_NB];
    __shared__ float2 Gs[BT_NB][BT_NB + 1];   // Gs[i][r] = G(r, i), upper part r < i
    for (int q = threadIdx.x; q < BT_NB * BT_NB; q += blockDim.x) {
        Tb[q] = make_float2(0.f, 0.f);
        const int r = q % BT_NB, i = q / BT_NB;
        float2 acc = make_float2(0.f, 0.f);
        if (r < i)
            for (int64_t s = 0; s < ks; ++s) acc = vadd(acc, G[(s * batch + b) * BT_NB * BT_NB + q]);
        Gs[i][r] = acc;
    }
    __syncthreads();
    for (int64_t i = 0; i < nbk; ++i) {
        const float2 ti = tb[j0 + i];
        if (threadIdx.x < i) tmp[threadIdx.x] = vmul(make_float2(-ti.x, -ti.y), Gs[i][threadIdx.x]);
        __syncthreads();
        if (threadIdx.x < i) {
            float2 s = make_float2(0.f, 0.f);
            for (int64_t q = threadIdx.x; q < i; ++q) s = vadd(s, vmul(Tb[threadIdx.x + q * BT_NB], tmp[q]));
            Tb[threadIdx.x + i * BT_NB] = s;
        }
        if (threadIdx.x == 0) Tb[i + i * BT_NB] = ti;
        __syncthreads();
    }
}

// A1: 128 rows (2l = Re W, 2l+1 = Im W) x 6 segments of Kp (rows r = j0 + kk of V)
__global__ void k_stage_bt1(const float2* __restrict__ A, int64_t lda, int64_t strideA, int64_t n, int64_t j0,
                            int64_t nbk, int64_t Kp, float* __restrict__ A1, int64_t a1Stride) {
    const int64_t b = blockIdx.z;
    const int64_t kk = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int l = blockIdx.y;
    if (kk >= Kp) return;
    float2 v = (l < nbk) ? bt_v(A + b * strideA, lda, n, j0 + l, j0 + kk) : make_float2(0.f, 0.f);
    float vrh, vrl, vih, vil;
    split2(v.x, vrh, vrl);
    split2(v.y, vih, vil);
    float* re = A1 + b * a1Stride + (2 * l) * 6 * Kp;
    float* im = re + 6 * Kp;
    // segments pair with X planes {hi.re, hi.im, lo.re, lo.im, hi.re, hi.im}
    re[kk] = vrh;          re[Kp + kk] = vih;
    re[2 * Kp + kk] = vrh; re[3 * Kp + kk] = vih;
    re[4 * Kp + kk] = vrl; re[5 * Kp + kk] = vil;
    im[kk] = -vih;          im[Kp + kk] = vrh;
    im[2 * Kp + kk] = -vih; im[3 * Kp + kk] = vrh;
    im[4 * Kp + kk] = -vil; im[5 * Kp + kk] = vrl;
}

// GEMM1 epilogue: W(l, c) = (row 2l, row 2l+1) of K-split partial z = b * ks + s
struct BtW1Epi {
    float2* W;
    int64_t nbk, iu;
    __device__ void operator()(int64_t z, int64_t row, int64_t col0, const float* v, int64_t M, int64_t N) const {
        const int64_t l = row >> 1;
        const bool keep = (row & 1) == 0 && l < nbk;
        float2* __restrict__ w = W + z * BT_NB * iu + l + col0 * BT_NB;   // partial z
        const int64_t nc = iu - col0;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
            const float im = __shfl_xor_sync(0xffffffffu, v[q], 1);
            if (keep && q < nc) w[q * BT_NB] = make_float2(v[q], im);
        }
    }
};

// A2: rows 2rr (Re X) / 2rr+1 (Im X) for r = j0 + rr, 6 segments of 64 (l)
__global__ void k_stage_bt2(const float2* __restrict__ A, int64_t lda, int64_t strideA, int64_t n, int64_t j0,
                            int64_t nbk, float* __restrict__ A2, int64_t a2Stride) {
    const int64_t b = blockIdx.y;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t rr = t / BT_NB;
    const int l = (int)(t - rr * BT_NB);
    if (j0 + rr >= n) return;
    float2 v = (l < nbk) ? bt_v(A + b * strideA, lda, n, j0 + l, j0 + rr) : make_float2(0.f, 0.f);
    float vrh, vrl, vih, vil;
    split2(v.x, vrh, vrl);
    split2(v.y, vih, vil);
    float* re = A2 + b * a2Stride + (2 * rr) * 6 * BT_NB;
    float* im = re + 6 * BT_NB;
    // segments pair with W2 parts {hi.re, hi.im, lo.re, lo.im, hi.re, hi.im}
    re[l] = vrh;           re[64 + l] = -vih;
    re[128 + l] = vrh;     re[192 + l] = -vih;
    re[256 + l] = vrl;     re[320 + l] = -vil;
    im[l] = vih;           im[64 + l] = vrh;
    im[128 + l] = vih;     im[192 + l] = vrh;
    im[256 + l] = vil;     im[320 + l] = vrl;
}

// B2: rows c of W2^T, 6 segments of 64 (l)
__global__ void k_stage_bt3(const float2* __restrict__ W2, int64_t iu, float* __restrict__ B2, int64_t b2Stride) {
    const int64_t b = blockIdx.y;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t c = t / BT_NB;
    const int l = (int)(t - c * BT_NB);
    if (c >= iu) return;
    const float2 w = W2[b * BT_NB * iu + l + c * BT_NB];
    float rh, rl, ih, il;
    split2(w.x, rh, rl);
    split2(w.y, ih, il);
    float* o = B2 + b * b2Stride + c * 6 * BT_NB;
    o[l] = rh;       o[64 + l] = ih;
    o[128 + l] = rl; o[192 + l] = il;
    o[256 + l] = rh; o[320 + l] = ih;
}

// GEMM2 epilogue: X(j0 + rr, c) -= D, re-split into the hi / lo planes.  The two lanes of a row
// pair split the 32 columns (even lane 0..15, odd lane 16..31).
struct BtXEpi {
    float* Xs;
    int64_t n4, iu, j0, n;
    __device__ void operator()(int64_t b, int64_t row, int64_t col0, const float* v, int64_t M, int64_t N) const {
        const int64_t rr = row >> 1, r = j0 + rr;
        const bool odd = (row & 1) != 0;
        const size_t P = (size_t)n4 * iu;
        float* __restrict__ X = Xs + b * 4 * P;
        float other[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) other[q] = __shfl_xor_sync(0xffffffffu, odd ? v[q] : v[16 + q], 1);
        if (row >= M || r >= n) return;
        const int h0 = odd ? 16 : 0;
        float hr[16], hi[16], lr[16], li[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int64_t c = col0 + h0 + q;
            const size_t o = (size_t)(c < iu ? c : 0) * n4 + r;
            hr[q] = X[o];
            hi[q] = X[P + o];
            lr[q] = X[2 * P + o];
            li[q] = X[3 * P + o];
        }
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            const int64_t c = col0 + h0 + q;
            if (c < iu) {
                const float dre = odd ? other[q] : v[q];
                const float dim = odd ? v[16 + q] : other[q];
                const size_t o = (size_t)c * n4 + r;
                const float xr = (hr[q] + lr[q]) - dre;
                const float xi = (hi[q] + li[q]) - dim;
                float h, l;
                split2(xr, h, l);
                X[o] = h;
                X[2 * P + o] = l;
                split2(xi, h, l);
                X[P + o] = h;
                X[3 * P + o] = l;
            }
        }
    }
};

int backtransform_tc(cudaStream_t st, MixedWs& ws, int64_t batch) {
    const int64_t n = ws.n, iu = ws.iu, n4 = ws.n4;
    const int64_t nrefl = n - 1;
    const int64_t nblocks = (nrefl + BT_NB - 1) / BT_NB;
    const int64_t lda = n, strideA = n * n;
    int64_t ksg_cap, ksw_cap;
    bt_split_caps(n, iu, batch, ksg_cap, ksw_cap);
    for (int64_t blk = nblocks - 1; blk >= 0; --blk) {
        const int64_t j0 = blk * BT_NB;
        const int64_t nbk = (nrefl - j0 < BT_NB) ? (nrefl - j0) : BT_NB;
        const int64_t Krows = n - j0;                      // rows j0 .. n-1
        const int64_t nkp = (Krows + 31) / 32;
        const int64_t Kp = nkp * 32;
        int64_t ksw = 1;
        // Gram (CUDA cores, FP32, split over K to fill the GPU) and compact-WY factor
        const int64_t kg_want = std::min<int64_t>(ksg_cap, (Krows + 255) / 256);
        const int64_t ksg = zg_ksplit_count(Krows, kg_want);
        FORGE_TRY((zgemm_launch_splitk<float2, KMAJOR, KMAJOR>(
            st, BT_NB, BT_NB, Krows, batch, kg_want, BtGA{ws.A32, lda, strideA, n, j0, nbk},
            BtGB{ws.A32, lda, strideA, n, j0, nbk}, StoreGramSplit{ws.G, batch})));
        k_larft32<<<(unsigned)batch, BT_NB, 0, st>>>(ws.G, ksg, batch, ws.tau, n, j0, nbk, ws.T);
        FORGE_LAUNCH_CHECK();
        // W = V^H X  (tensor cores)
        k_stage_bt1<<<dim3((unsigned)((Kp + 255) / 256), BT_NB, (unsigned)batch), 256, 0, st>>>(
            ws.A32, lda, strideA, n, j0, nbk, Kp, ws.A1, 2 * BT_NB * 6 * ws.Kp);
        FORGE_LAUNCH_CHECK();
        {
            TcOperand A{ws.A1, 2 * BT_NB, 6 * Kp, 6 * Kp, 2 * BT_NB * 6 * ws.Kp, batch};
            TcKMap ka = tc_kmap_plain(6 * Kp);
            TcOperand B{ws.Xs, iu, n4, n4, n4 * iu, 4 * batch};
            TcKMap kb{};
            kb.nkp = (int32_t)nkp;
            kb.nseg = 6;
            kb.koff = (int32_t)j0;
            kb.zbatch = 4;
            const int32_t zs[6] = {0, 1, 2, 3, 0, 1};
            for (int q = 0; q < 6; ++q) kb.zsel[q] = zs[q];
            // split K so that the (1 x iu/128 x batch) tile grid fills the GPU
            const int want = (int)std::min<int64_t>(ksw_cap, std::max<int64_t>(1, 6 * nkp / 8));
            ksw = tc_ksplit_count(6 * nkp, want);
            FORGE_TRY(tc_gemm_tf32_mapped(st, A, ka, B, kb, batch, 0, BtW1Epi{ws.Wb, nbk, iu}, ws.err, want));
        }
        // W2 = T W (CUDA cores; W summed over its K-split partials on load)
        FORGE_TRY((zgemm_launch<float2, IMAJOR, KMAJOR, false>(st, BT_NB, iu, BT_NB, batch, TWa{ws.T, nbk},
                                                                TWb{ws.Wb, nbk, iu, ksw},
                                                                StoreF2{ws.W2, BT_NB, BT_NB * iu})));
        // X(j0:, :) -= V W2  (tensor cores)
        k_stage_bt2<<<dim3((unsigned)((Krows * BT_NB + 255) / 256), (unsigned)batch), 256, 0, st>>>(
            ws.A32, lda, strideA, n, j0, nbk, ws.A2, 2 * n * 6 * BT_NB);
        FORGE_LAUNCH_CHECK();
        k_stage_bt3<<<dim3((unsigned)((iu * BT_NB + 255) / 256), (unsigned)batch), 256, 0, st>>>(
            ws.W2, iu, ws.B2, iu * 6 * BT_NB);
        FORGE_LAUNCH_CHECK();
        {
            TcOperand A{ws.A2, 2 * Krows, 6 * BT_NB, 6 * BT_NB, 2 * n * 6 * BT_NB, batch};
            TcOperand B{ws.B2, iu, 6 * BT_NB, 6 * BT_NB, iu * 6 * BT_NB, batch};
            FORGE_TRY(tc_gemm_tf32_mapped(st, A, tc_kmap_plain(6 * BT_NB), B, tc_kmap_plain(6 * BT_NB), batch, 0,
                                          BtXEpi{ws.Xs, n4, iu, j0, n}, ws.err));
        }
    }
    return 0;
}

// ---------------------------------------------------------------- driver
int eig_mixed(cudaStream_t st, EigArgs& g, void* mixed_ws) {
    MixedWs ws{};
    ws.n = g.n;
    ws.iu = g.iu;
    ws.B = g.batch;
    Carve c{static_cast<char*>(mixed_ws)};
    carve(ws, c);
    const int64_t n = g.n, iu = g.iu, batch = g.batch;
    FORGE_CUDA(cudaMemsetAsync(ws.err, 0, sizeof(int), st));
    k_h_to_f32<<<1216, 256, 0, st>>>(g.A, ws.A32, (size_t)batch * n * n);
    FORGE_LAUNCH_CHECK();
    TrdArgs<float> a;
    a.A = ws.A32;
    a.lda = n;
    a.strideA = n * n;
    a.n = n;
    a.d = g.d;
    a.e = g.e;
    a.tau = ws.tau;
    a.W = ws.W;
    a.Yrow = ws.Yrow;
    a.Ycol = ws.Ycol;
    a.ystride = ws.nblk * n;
    a.Spart = ws.Spart;
    a.sstride = ws.nrb * 2 * TRD_NB;
    a.part = ws.part;
    a.pstride = ws.pstride;
    a.scal = ws.scal;
    a.cnt = ws.cnt;
    a.her2k = her2k_tc;
    a.her2k_user = &ws;
    FORGE_CUDA(cudaMemsetAsync(ws.cnt, 0, sizeof(unsigned) * 4 * batch, st));
    FORGE_TRY(tridiagonalize<float>(st, a, batch));
    // eigenvalues of T: FP32 bisection, then FP64 bisection from the FP32 bracket
    EigArgs ge = g;
    ge.bisect_f32 = 1;
    FORGE_TRY(tridiag_eigvecs(st, ge));
    dim3 gz((unsigned)((ws.n4 + 31) / 32), (unsigned)((iu + 31) / 32), (unsigned)batch);
    k_z_to_planes<<<gz, dim3(32, 8), 0, st>>>(g.Z, n, ws.n4, iu, ws.Xs);
    FORGE_LAUNCH_CHECK();
    prof_begin(ST_BACKTRANSFORM);
    FORGE_TRY(backtransform_tc(st, ws, batch));
    prof_end(ST_BACKTRANSFORM, batch * (double)n * iu * 16.0 * 2.0, batch * 3.0 * 8.0 * (double)n * n * iu);
    // FP64 copies of the first iu_out columns (the planes keep all iu for the eigenpair refinement)
    const int64_t iu_out = (g.iu_out > 0 && g.iu_out < iu) ? g.iu_out : iu;
    k_planes_to_x<<<dim3(1216, (unsigned)batch), 256, 0, st>>>(ws.Xs, n, ws.n4, iu, iu_out, g.X, g.ldx, g.strideX);
    FORGE_LAUNCH_CHECK();
    k_normalize_cols<<<dim3((unsigned)iu_out, (unsigned)batch), 256, 0, st>>>(g.X, n, iu_out, g.ldx, g.strideX);
    FORGE_LAUNCH_CHECK();
    int herr = 0;
    FORGE_CUDA(cudaMemcpyAsync(&herr, ws.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    FORGE_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        set_error(FORGE_ERR_TIMEOUT, "tcgen05 GEMM: a bounded mbarrier wait gave up");
        return FORGE_ERR_TIMEOUT;
    }
    return 0;
}

}  // namespace forge
