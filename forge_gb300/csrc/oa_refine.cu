// Eigenpair refinement of the mixed-precision eigen-solver on the tensor cores: one step of
// Ogita & Aishima's iterative refinement for Hermitian eigenproblems (T. Ogita, K. Aishima,
// "Iterative refinement for symmetric eigenvalue problems", Japan J. Indust. Appl. Math. 35
// (2018) 1007-1035), written in its residual form.
//
// The reference solves every H(k) with FP64 zheevr (LapackRoutines.f90:414-426).  The mixed
// solver gives FP32-accurate eigenpairs of all n eigenvalues; this step makes the first iu of
// them FP64-accurate.  Per matrix, with lam the mixed eigenvalues (ascending):
//   W    = H X_j - X_j lam_j            (j < iu)   error-free sliced product on the tensor cores:
//                                       |W| ~ 1e-6 |H| and W must be exact to ~2^-40 |H||X|
//   C    = X_all^H W                               TF32 hi/lo products (W is small: FP32 accuracy
//                                                   of C is enough)
//   E_ij = C_ij / (lam_j - lam_i)       if |lam_j - lam_i| > delta
//        = -(x_i^H x_j) / 2             otherwise (i != j; FP64 overlaps): orthogonalisation only
//   X_j += X_all E_:j                              TF32 hi/lo products, accumulated into FP64 X
//   lam_j += x_j^H w_j                             FP64 (the Rayleigh quotient of the input x_j)
// and the refined columns are renormalised in FP64.  The correction uses every eigenvector of
// H, so mixing with eigenvectors above iu is removed too.  Pairs closer than delta keep their
// mixing (both occupied: no effect on the density matrix; around the Fermi level the FP64
// window Rayleigh-Ritz that follows resolves them).
//
// The residual product H X runs as real GEMMs over integer slices (Ozaki et al., Numer.
// Algorithms 59 (2012)): every row of H and column of X is scaled by a power of two to |v| < 1
// and cut into slices v = sum_s v_s 2^-(8 + 9 s) with integer |v_s| <= 256; slice products with
// s + t <= depth are summed by the exact-block mode of the tcgen05 GEMM (integer blocks of 256
// products, double-float accumulation), which keeps ~2^-(16 + 9 (depth + 1)) of |H||X|.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cvec.cuh"
#include "forge_internal.cuh"
#include "tc_gemm.cuh"

namespace forge {

constexpr int OA_SLICES = 5;         // slices per operand (depth <= 4 uses all five)
constexpr int OA_CLUSTER_RADIUS = 64;

namespace {

inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

__device__ inline float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Fills the strict upper triangle of every H(k) with the conjugate of its lower triangle.
// 32 x 32 tiles (tr, tc), tc >= tr; reads and writes are coalesced along rows.
__global__ void k_herm_fill(double2* __restrict__ H, int64_t n) {
    const int64_t tr = blockIdx.y, tc = blockIdx.x;
    if (tc < tr) return;
    __shared__ double2 t[32][33];
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int64_t r = tc * 32 + threadIdx.x, c = tr * 32 + yy;   // source (lower): row r, column c
        t[yy][threadIdx.x] = (r < n && c < n) ? H[r + c * n] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int64_t r = tr * 32 + threadIdx.x, c = tc * 32 + yy;   // destination (upper): row r < c
        if (r < n && c < n && r < c) {
            const double2 v = t[threadIdx.x][yy];
            H[r + c * n] = make_double2(v.x, -v.y);
        }
    }
}

// Slices of one column per CTA.  mode 0 (H -> rows of the A operand): column i of the full
// Hermitian H is conj(row i), so planes 0..S-1 hold the slices of Re H(i, k) = Re H(k, i) and
// planes S..2S-1 those of Im H(i, k) = -Im H(k, i).  mode 1 (X -> rows of the B operand):
// planes Re (0..S-1), Im (S..2S-1), -Im (2S..3S-1).  Plane p of the output:
// out + p * pstride + col * pitch + row; the column's power-of-two scale goes to expo[col].
__global__ void __launch_bounds__(256) k_oa_slice(const double2* __restrict__ src, int64_t ld, int64_t nrows,
                                                  int mode, float* __restrict__ out, int64_t pitch, int64_t pstride,
                                                  int* __restrict__ expo) {
    const int64_t col = blockIdx.x;
    const double2* s = src + col * ld;
    double m = 0.0;
    for (int64_t r = threadIdx.x; r < nrows; r += blockDim.x) m = fmax(m, fmax(fabs(s[r].x), fabs(s[r].y)));
    __shared__ double red[8];
    m = warp_max_d(m);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
        t = warp_max_d(t);
        if (threadIdx.x == 0) red[0] = t;
    }
    __syncthreads();
    int e = 0;
    if (red[0] > 0.0) frexp(red[0], &e);   // red[0] < 2^e
    if (threadIdx.x == 0) expo[col] = e;
    constexpr int S = OA_SLICES;
    for (int64_t r = threadIdx.x; r < nrows; r += blockDim.x) {
        double a[2] = {ldexp(s[r].x, -e), ldexp(s[r].y, -e)};   // |a| < 1, exact
        if (mode == 0) a[1] = -a[1];                            // row i of H = conj(column i)
        for (int part = 0; part < 2; ++part) {
            double t = a[part] * 256.0;
            for (int q = 0; q < S; ++q) {
                const double v = rint(t);                        // |v| <= 256
                t = (t - v) * 512.0;                             // exact: the remainder has <= 53 bits
                const int64_t o = col * pitch + r;
                const float fv = (float)v;
                out[(part * S + q) * pstride + o] = fv;
                if (mode == 1 && part == 1) out[(2 * S + q) * pstride + o] = -fv;
            }
        }
    }
}

// W = H X - X lam (one part per launch), written as TF32 hi/lo planes of the B operand of C:
// plane 0 Re hi, 1 Re lo, 2 Im hi, 3 Im lo, 4 -Re hi, 5 -Re lo; element (k, j) at j * pitch + k.
struct OaWEpi {
    const int *eA, *eB;
    const double2* X;
    int64_t ldx;
    const double* lam;
    float* Wp;
    int64_t pitch, pstride;
    int part;
    __device__ void operator()(int64_t, int64_t row, int64_t col0, const double* v, int64_t M, int64_t N) const {
        if (row >= M) return;
        const int ea = eA[row];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
            const int64_t j = col0 + q;
            if (j >= N) continue;
            const double y = ldexp(v[q], ea + eB[j]);
            const double2 x = X[row + j * ldx];
            const double w = y - (part ? x.y : x.x) * lam[j];
            const float hi = tf32_rna((float)w);
            const float lo = (float)(w - (double)hi);
            const int64_t o = j * pitch + row;
            if (part == 0) {
                Wp[o] = hi;
                Wp[pstride + o] = lo;
                Wp[4 * pstride + o] = -hi;
                Wp[5 * pstride + o] = -lo;
            } else {
                Wp[2 * pstride + o] = hi;
                Wp[3 * pstride + o] = lo;
            }
        }
    }
};

// E_ij = C_ij / (lam_j - lam_i) for separated pairs, 0 for i == j and cluster pairs (filled by
// k_oa_cluster); TF32 hi/lo planes of the B operand of the update: 0 Re hi, 1 Re lo, 2 Im hi,
// 3 Im lo, 4 -Im hi, 5 -Im lo; element (i, j) at j * pitch + i.
struct OaCEpi {
    const double* lam;
    double delta;
    float* Ep;
    int64_t pitch, pstride;
    int part;
    __device__ void operator()(int64_t, int64_t row, int64_t col0, const float* v, int64_t M, int64_t N) const {
        if (row >= M) return;
        const double li = lam[row];
#pragma unroll
        for (int q = 0; q < 32; ++q) {
            const int64_t j = col0 + q;
            if (j >= N) continue;
            const double d = lam[j] - li;
            const double e = (j != row && fabs(d) > delta) ? (double)v[q] / d : 0.0;
            const float hi = tf32_rna((float)e);
            const float lo = (float)(e - (double)hi);
            const int64_t o = j * pitch + row;
            if (part == 0) {
                Ep[o] = hi;
                Ep[pstride + o] = lo;
            } else {
                Ep[2 * pstride + o] = hi;
                Ep[3 * pstride + o] = lo;
                Ep[4 * pstride + o] = -hi;
                Ep[5 * pstride + o] = -lo;
            }
        }
    }
};

// X(r, j) += the update of one part
struct OaUEpi {
    double2* X;
    int64_t ldx;
    int part;
    __device__ void operator()(int64_t, int64_t row, int64_t col0, const float* v, int64_t M, int64_t N) const {
        if (row >= M) return;
#pragma unroll
        for (int q = 0; q < 32; ++q) {
            const int64_t j = col0 + q;
            if (j >= N) continue;
            double2* p = X + row + j * ldx;
            if (part == 0)
                p->x += (double)v[q];
            else
                p->y += (double)v[q];
        }
    }
};

__device__ inline double2 plane_x(const float* Xs, int64_t P, int64_t o) {
    return make_double2((double)Xs[o] + (double)Xs[2 * P + o], (double)Xs[P + o] + (double)Xs[3 * P + o]);
}

// Cluster pairs of column j (|lam_i - lam_j| <= delta, i != j, |i - j| <= OA_CLUSTER_RADIUS):
// E_ij = -(x_i^H x_j) / 2 from the FP32-accurate planes, summed in FP64.  One CTA per column.
__global__ void __launch_bounds__(256) k_oa_cluster(const float* __restrict__ Xs, int64_t n4, int64_t nall,
                                                    int64_t n, const double* __restrict__ lam, double delta,
                                                    float* __restrict__ Ep, int64_t pitch, int64_t pstride) {
    const int64_t j = blockIdx.x;
    const int64_t P = n4 * nall;
    int64_t lo = j, hi = j;
    while (lo > 0 && j - lo < OA_CLUSTER_RADIUS && lam[j] - lam[lo - 1] <= delta) --lo;
    while (hi + 1 < nall && hi - j < OA_CLUSTER_RADIUS && lam[hi + 1] - lam[j] <= delta) ++hi;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t i = lo + warp; i <= hi; i += 8) {
        if (i == j) continue;
        double2 acc = make_double2(0.0, 0.0);
        for (int64_t k = lane; k < n; k += 32) {
            const double2 a = plane_x(Xs, P, i * n4 + k), b = plane_x(Xs, P, j * n4 + k);
            acc.x += a.x * b.x + a.y * b.y;
            acc.y += a.x * b.y - a.y * b.x;
        }
        acc = warp_sum(acc);
        if (lane == 0) {
            const double er = -0.5 * acc.x, ei = -0.5 * acc.y;
            const int64_t o = j * pitch + i;
            float h = tf32_rna((float)er);
            Ep[o] = h;
            Ep[pstride + o] = (float)(er - (double)h);
            h = tf32_rna((float)ei);
            const float l = (float)(ei - (double)h);
            Ep[2 * pstride + o] = h;
            Ep[3 * pstride + o] = l;
            Ep[4 * pstride + o] = -h;
            Ep[5 * pstride + o] = -l;
        }
    }
}

// lam_out(j) = lam(j) + Re(x_j^H w_j) in FP64 (x_j unit-normalised).  One CTA per column.
__global__ void __launch_bounds__(256) k_oa_diag(const double2* __restrict__ X, int64_t ldx, int64_t n,
                                                 const float* __restrict__ Wp, int64_t pitch, int64_t pstride,
                                                 const double* __restrict__ lam, double* __restrict__ lam_out) {
    const int64_t j = blockIdx.x;
    double s = 0.0;
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) {
        const int64_t o = j * pitch + r;
        const double wr = (double)Wp[o] + (double)Wp[pstride + o];
        const double wi = (double)Wp[2 * pstride + o] + (double)Wp[3 * pstride + o];
        const double2 x = X[r + j * ldx];
        s += x.x * wr + x.y * wi;
    }
    __shared__ double red[8];
    s = warp_sum_d(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w];
        lam_out[j] = lam[j] + t;
    }
}

// Xs planes (column-major: element (r, i) at i * n4 + r) -> XT planes (element (r, i) at
// r * pitchT + i), four planes.  32 x 32 tiles: blockIdx.x over i, blockIdx.y over r.
__global__ void k_oa_transpose(const float* __restrict__ Xs, int64_t n4, int64_t nall, int64_t n,
                               float* __restrict__ XT, int64_t pitchT) {
    __shared__ float t[4][32][33];
    const int64_t i0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int64_t P = n4 * nall, PT = n * pitchT;
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int64_t i = i0 + yy, r = r0 + threadIdx.x;
#pragma unroll
        for (int p = 0; p < 4; ++p) t[p][yy][threadIdx.x] = (i < nall && r < n) ? Xs[p * P + i * n4 + r] : 0.f;
    }
    __syncthreads();
    for (int yy = threadIdx.y; yy < 32; yy += blockDim.y) {
        const int64_t r = r0 + yy, i = i0 + threadIdx.x;
        if (r < n && i < nall) {
#pragma unroll
            for (int p = 0; p < 4; ++p) XT[p * PT + r * pitchT + i] = t[p][threadIdx.x][yy];
        }
    }
}

__global__ void k_normalize(double2* __restrict__ X, int64_t n, int64_t ldx) {
    const int64_t c = blockIdx.x;
    double2* x = X + c * ldx;
    double s = 0.0;
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) s += x[r].x * x[r].x + x[r].y * x[r].y;
    __shared__ double red[8];
    s = warp_sum_d(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t += red[w];
        red[0] = t;
    }
    __syncthreads();
    const double scl = red[0] > 0.0 ? 1.0 / sqrt(red[0]) : 1.0;
    for (int64_t r = threadIdx.x; r < n; r += blockDim.x) x[r] = make_double2(x[r].x * scl, x[r].y * scl);
}

struct OaLayout {
    int64_t pitch, K256, nslab, nA, nB, nW, nE, nT;
    float *A, *B, *W, *E, *T;
    int *eA, *eB;
};

OaLayout oa_layout(int64_t n, int64_t iu, void* base) {
    OaLayout L{};
    L.pitch = round_up(n, 4);
    L.K256 = round_up(n, 256);
    constexpr int S = OA_SLICES;
    L.nA = 2 * S * n * L.pitch;
    L.nB = 3 * S * iu * L.pitch;
    L.nW = 6 * iu * L.pitch;
    L.nE = 6 * iu * L.pitch;
    L.nT = 4 * n * L.pitch;
    char* p = static_cast<char*>(base);
    auto take = [&](size_t bytes) {
        char* q = p;
        p += round_up((int64_t)bytes, 256);
        return q;
    };
    L.A = (float*)take(L.nA * 4);
    L.B = (float*)take(L.nB * 4);
    L.W = (float*)take(L.nW * 4);
    L.E = (float*)take(L.nE * 4);
    L.T = (float*)take(L.nT * 4);
    L.eA = (int*)take(n * 4);
    L.eB = (int*)take(iu * 4);
    L.nslab = (int64_t)(p - static_cast<char*>(base));
    return L;
}

}  // namespace

size_t oa_workspace_bytes(int64_t n, int64_t iu) { return (size_t)oa_layout(n, iu, nullptr).nslab + 256; }

// Refines columns 0..iu-1 of X (FP64, unit-normalised, ldx, strideX per matrix) and their eigenvalues
// for each of the batch matrices: H (FP64, lower triangles; the upper triangles are filled here), Xs
// (the mixed solve's TF32 hi/lo planes of all nall = n eigenvectors, four planes of n4 x nall per
// matrix), lam (nall eigenvalues per matrix, ascending).  The refined eigenvalues go to
// w_out + b * w_stride.  depth: slice products s + t <= depth of the residual (3 or 4).
int oa_refine(cudaStream_t st, double2* H, int64_t strideH, const float* Xs, int64_t n4, int64_t nall,
              const double* lam, int64_t n, int64_t iu, int64_t batch, double2* X, int64_t ldx, int64_t strideX,
              double* w_out, int64_t w_stride, void* ws, int* err, double delta, int depth) {
    if (iu <= 0 || batch <= 0) return 0;
    if (nall != n || iu > nall || depth < 1 || depth > OA_SLICES - 1 || n4 < n || (n4 % 4)) {
        set_error(FORGE_ERR_ARG, "oa_refine: needs all n eigenvectors (nall=%lld n=%lld), iu <= n, depth 1..%d",
                  (long long)nall, (long long)n, OA_SLICES - 1);
        return FORGE_ERR_ARG;
    }
    OaLayout L = oa_layout(n, iu, ws);
    constexpr int S = OA_SLICES;
    // slice pairs (s, t), s + t <= depth, and their scale 2^-(16 + 9 (s + t))
    std::vector<std::pair<int, int>> pairs;
    for (int d = 0; d <= depth; ++d)
        for (int s = 0; s <= d; ++s) pairs.push_back({s, d - s});
    const int nseg = 2 * (int)pairs.size();
    if (nseg > TC_MAXSEG) {
        set_error(FORGE_ERR_ARG, "oa_refine: %d segments exceed %d", nseg, TC_MAXSEG);
        return FORGE_ERR_ARG;
    }
    const int32_t nkp256 = (int32_t)(L.K256 / 32);
    auto wmap = [&](int part, TcKMap& ka, TcKMap& kb) {
        ka = TcKMap{};
        kb = TcKMap{};
        ka.nkp = kb.nkp = nkp256;
        ka.nseg = kb.nseg = nseg;
        ka.zbatch = kb.zbatch = 0;
        int q = 0;
        for (auto [s, t] : pairs) {
            const int8_t sc = (int8_t)(16 + 9 * (s + t));
            // part 0: Re(HX) = Re H Re X - Im H Im X; part 1: Im(HX) = Re H Im X + Im H Re X
            ka.zsel[q] = s;
            kb.zsel[q] = part == 0 ? t : S + t;
            ka.sexp[q++] = sc;
            ka.zsel[q] = S + s;
            kb.zsel[q] = part == 0 ? 2 * S + t : t;
            ka.sexp[q++] = sc;
        }
    };
    auto cmap = [&](const int32_t* za, const int32_t* zb, int64_t K, TcKMap& ka, TcKMap& kb) {
        ka = TcKMap{};
        kb = TcKMap{};
        ka.nkp = kb.nkp = (int32_t)((K + 31) / 32);
        ka.nseg = kb.nseg = 6;
        for (int q = 0; q < 6; ++q) {
            ka.zsel[q] = za[q];
            kb.zsel[q] = zb[q];
        }
    };
    const double nd = (double)n, iud = (double)iu;
    for (int64_t b = 0; b < batch; ++b) {
        double2* Hb = H + b * strideH;
        const float* Xsb = Xs + b * 4 * n4 * nall;
        const double* lamb = lam + b * nall;
        double2* Xb = X + b * strideX;
        double* wb = w_out + b * w_stride;
        prof_begin(ST_OA);
        const unsigned nt = (unsigned)((n + 31) / 32);
        k_herm_fill<<<dim3(nt, nt), dim3(32, 8), 0, st>>>(Hb, n);
        FORGE_LAUNCH_CHECK();
        k_oa_slice<<<(unsigned)n, 256, 0, st>>>(Hb, n, n, 0, L.A, L.pitch, n * L.pitch, L.eA);
        FORGE_LAUNCH_CHECK();
        k_oa_slice<<<(unsigned)iu, 256, 0, st>>>(Xb, ldx, n, 1, L.B, L.pitch, iu * L.pitch, L.eB);
        FORGE_LAUNCH_CHECK();
        prof_end(ST_OA, nd * nd * 16.0 * 2.0 + nd * nd * 4.0 * 2 * S + nd * iud * (16.0 + 4.0 * 3 * S), 0.0);
        // W = H X - X lam (sliced, exact blocks)
        prof_begin(ST_OA_GEMM);
        for (int part = 0; part < 2; ++part) {
            TcKMap ka, kb;
            wmap(part, ka, kb);
            TcOperand A{L.A, n, n, L.pitch, n * L.pitch, 2 * S};
            TcOperand B{L.B, iu, n, L.pitch, iu * L.pitch, 3 * S};
            FORGE_TRY((tc_gemm_tf32_mapped<OaWEpi, 8, true>(
                st, A, ka, B, kb, 1, 0, OaWEpi{L.eA, L.eB, Xb, ldx, lamb, L.W, L.pitch, iu * L.pitch, part}, err)));
        }
        prof_end(ST_OA_GEMM, nd * iud * 16.0 * 2.0 + nd * nd * 16.0,
                 (double)pairs.size() * 8.0 * nd * nd * iud);
        prof_begin(ST_OA);
        k_oa_diag<<<(unsigned)iu, 256, 0, st>>>(Xb, ldx, n, L.W, L.pitch, iu * L.pitch, lamb, wb);
        FORGE_LAUNCH_CHECK();
        // C = X_all^H W -> E (separated pairs)
        {
            const int32_t za_r[6] = {0, 0, 2, 1, 1, 3}, zb_r[6] = {0, 1, 0, 2, 3, 2};
            const int32_t za_i[6] = {0, 0, 2, 1, 1, 3}, zb_i[6] = {2, 3, 2, 4, 5, 4};
            TcOperand A{Xsb, nall, n, n4, n4 * nall, 4};
            TcOperand B{L.W, iu, n, L.pitch, iu * L.pitch, 6};
            TcKMap ka, kb;
            cmap(za_r, zb_r, n, ka, kb);
            FORGE_TRY(tc_gemm_tf32_mapped(st, A, ka, B, kb, 1, 0,
                                          OaCEpi{lamb, delta, L.E, L.pitch, iu * L.pitch, 0}, err));
            cmap(za_i, zb_i, n, ka, kb);
            FORGE_TRY(tc_gemm_tf32_mapped(st, A, ka, B, kb, 1, 0,
                                          OaCEpi{lamb, delta, L.E, L.pitch, iu * L.pitch, 1}, err));
        }
        k_oa_cluster<<<(unsigned)iu, 256, 0, st>>>(Xsb, n4, nall, n, lamb, delta, L.E, L.pitch, iu * L.pitch);
        FORGE_LAUNCH_CHECK();
        // X_j += X_all E
        k_oa_transpose<<<dim3((unsigned)((nall + 31) / 32), nt), dim3(32, 8), 0, st>>>(Xsb, n4, nall, n, L.T,
                                                                                       L.pitch);
        FORGE_LAUNCH_CHECK();
        {
            const int32_t za_r[6] = {0, 0, 2, 1, 1, 3}, zb_r[6] = {0, 1, 0, 4, 5, 4};
            const int32_t za_i[6] = {0, 0, 2, 1, 1, 3}, zb_i[6] = {2, 3, 2, 0, 1, 0};
            TcOperand A{L.T, n, nall, L.pitch, n * L.pitch, 4};
            TcOperand B{L.E, iu, nall, L.pitch, iu * L.pitch, 6};
            TcKMap ka, kb;
            cmap(za_r, zb_r, nall, ka, kb);
            FORGE_TRY(tc_gemm_tf32_mapped(st, A, ka, B, kb, 1, 0, OaUEpi{Xb, ldx, 0}, err));
            cmap(za_i, zb_i, nall, ka, kb);
            FORGE_TRY(tc_gemm_tf32_mapped(st, A, ka, B, kb, 1, 0, OaUEpi{Xb, ldx, 1}, err));
        }
        k_normalize<<<(unsigned)iu, 256, 0, st>>>(Xb, n, ldx);
        FORGE_LAUNCH_CHECK();
        prof_end(ST_OA, nd * nd * 4.0 * 4.0 * 2.0 + 2.0 * nd * iud * (16.0 + 24.0),
                 2.0 * 3.0 * 8.0 * nd * nd * iud);
    }
    return 0;
}

}  // namespace forge
