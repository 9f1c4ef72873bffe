// Eigenpairs 1..iu of the real symmetric tridiagonal T (d, e) and back-transformation
// X = Q Z, batched over k.
//
// zheevr with RANGE='I' and IU < N (LapackRoutines.f90:414-426) computes the
// eigenvalues by bisection (dstebz) and the vectors by inverse iteration (zstein);
// this file restates that route for the GPU:
//   k_gersh     : Gershgorin interval, 1-norm and pivmin per matrix;
//   k_bisect    : one thread per eigenvalue, Sturm counts in FP64 (dlaebz rules);
//   k_clusters  : groups consecutive eigenvalues closer than ortol;
//   k_invit     : one thread per cluster: LU of T - lambda I with partial pivoting
//                 (dlagtf), perturbed back-substitution (dlagts, job=-1), modified
//                 Gram-Schmidt against the earlier members of the cluster;
//   back-transform: Q applied in compact-WY blocks (zlarft forward/columnwise), two
//                 GEMMs per block on the chosen engine.
// ortol is tighter than zstein's 1e-3*||T||_1 (which groups a whole dense spectrum
// into one serial cluster); with ortol = 1e-7*||T||_1 the vector error bound
// eps*||T||/gap stays below 1e-8 outside clusters.
#include <algorithm>
#include <cfloat>
#include "cvec.cuh"
#include "eig.cuh"
#include "zgemm_engine.cuh"

namespace forge {

constexpr double kEps = 1.1102230246251565e-16;    // dlamch('E')
constexpr double kSafmin = 2.2250738585072014e-308; // dlamch('S')

__global__ void k_gersh(const double* __restrict__ d, const double* __restrict__ e, int64_t n, double* __restrict__ info) {
    // one CTA (256 threads) per matrix; info[b*8 + 0..4] = gl, gu, onenrm, pivmin, tnorm
    const int64_t b = blockIdx.x;
    const double* D = d + b * n;
    const double* E = e + b * n;
    double gl = 1e300, gu = -1e300, nrm = 0.0, emax = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        double em = (i > 0) ? fabs(E[i - 1]) : 0.0;
        double ep = (i < n - 1) ? fabs(E[i]) : 0.0;
        gl = fmin(gl, D[i] - em - ep);
        gu = fmax(gu, D[i] + em + ep);
        nrm = fmax(nrm, fabs(D[i]) + em + ep);
        if (i < n - 1) emax = fmax(emax, E[i] * E[i]);
    }
    __shared__ double s[4][256];
    s[0][threadIdx.x] = gl;
    s[1][threadIdx.x] = gu;
    s[2][threadIdx.x] = nrm;
    s[3][threadIdx.x] = emax;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s[0][threadIdx.x] = fmin(s[0][threadIdx.x], s[0][threadIdx.x + o]);
            s[1][threadIdx.x] = fmax(s[1][threadIdx.x], s[1][threadIdx.x + o]);
            s[2][threadIdx.x] = fmax(s[2][threadIdx.x], s[2][threadIdx.x + o]);
            s[3][threadIdx.x] = fmax(s[3][threadIdx.x], s[3][threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double pivmin = kSafmin * fmax(1.0, s[3][0]);
        double tnorm = fmax(fabs(s[0][0]), fabs(s[1][0]));
        const double fudge = 2.1, ulp = 2.0 * kEps;
        double g0 = s[0][0] - fudge * tnorm * ulp * n - fudge * 2.0 * pivmin;
        double g1 = s[1][0] + fudge * tnorm * ulp * n + fudge * 2.0 * pivmin;
        info[b * 8 + 0] = g0;
        info[b * 8 + 1] = g1;
        info[b * 8 + 2] = s[2][0];
        info[b * 8 + 3] = pivmin;
        info[b * 8 + 4] = tnorm;
    }
}

// number of eigenvalues <= x (dlaebz Sturm count)
__device__ inline int64_t sturm(const double* D, const double* E, int64_t n, double x, double pivmin) {
    double q = D[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    int64_t cnt = (q <= 0.0) ? 1 : 0;
    for (int64_t i = 1; i < n; ++i) {
        const double e = E[i - 1];
        q = D[i] - e * e / q - x;
        if (fabs(q) < pivmin) q = -pivmin;
        cnt += (q <= 0.0) ? 1 : 0;
    }
    return cnt;
}

// With a FP32 estimate in w (from k_bisect_f32) the FP64 bisection starts from the bracket
// w[j] -/+ 8 eps_32 ||T|| when the FP64 Sturm counts confirm that it holds eigenvalue j (about 33
// FP64 steps instead of 54), else from the Gershgorin interval.
__global__ void k_bisect(const double* __restrict__ d, const double* __restrict__ e, int64_t n, int64_t iu,
                         const double* __restrict__ info, double* __restrict__ w, int from_estimate, double rtol_abs) {
    const int64_t b = blockIdx.y;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= iu) return;
    const double* D = d + b * n;
    const double* E = e + b * n;
    double lo = info[b * 8 + 0], hi = info[b * 8 + 1];
    const double pivmin = info[b * 8 + 3];
    if (from_estimate) {
        const double x = w[b * iu + j], delta = 8.0 * (double)FLT_EPSILON * info[b * 8 + 4];
        const double l2 = fmax(lo, x - delta), h2 = fmin(hi, x + delta);
        if (l2 < h2 && sturm(D, E, n, l2, pivmin) < j + 1 && sturm(D, E, n, h2, pivmin) >= j + 1) {
            lo = l2;
            hi = h2;
        }
    }
    const double rtol = 4.0 * kEps;
    // rtol_abs > 0 (mixed path): stop at rtol_abs ||T||, far below the FP32 error of T itself
    const double atol = rtol_abs * info[b * 8 + 4];
    for (int it = 0; it < 256; ++it) {
        double width = hi - lo;
        double tol = fmax(fmax(fmax(kSafmin, pivmin), rtol * fmax(fabs(lo), fabs(hi))), atol);
        if (width <= tol) break;
        double mid = 0.5 * (lo + hi);
        if (sturm(D, E, n, mid, pivmin) >= j + 1)
            hi = mid;
        else
            lo = mid;
    }
    w[b * iu + j] = 0.5 * (lo + hi);
}

// FP32 copies of the tridiagonal for the FP32 bisection: tf[b][0..n) = d, tf[b][n..2n) = e^2
__global__ void k_tri_to_f32(const double* __restrict__ d, const double* __restrict__ e, int64_t n,
                             float* __restrict__ tf) {
    const int64_t b = blockIdx.y;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        tf[b * 2 * n + i] = (float)d[b * n + i];
        const double ei = (i < n - 1) ? e[b * n + i] : 0.0;
        tf[b * 2 * n + n + i] = (float)(ei * ei);
    }
}

// Sturm count in FP32 (the count is exact for a tridiagonal within a few FP32 ulps of T)
__device__ inline int sturm_f32(const float* __restrict__ D, const float* __restrict__ E2, int n, float x,
                                float pivmin) {
    float q = D[0] - x;
    if (fabsf(q) < pivmin) q = -pivmin;
    int cnt = (q <= 0.f) ? 1 : 0;
    for (int i = 1; i < n; ++i) {
        q = (D[i] - x) - __fdividef(E2[i - 1], q);
        if (fabsf(q) < pivmin) q = -pivmin;
        cnt += (q <= 0.f) ? 1 : 0;
    }
    return cnt;
}

// eigenvalue j by bisection to FP32 accuracy (about 24 steps instead of 54 in FP64)
__global__ void k_bisect_f32(const float* __restrict__ tf, int64_t n, int64_t iu, const double* __restrict__ info,
                             double* __restrict__ w) {
    const int64_t b = blockIdx.y;
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= iu) return;
    const float* D = tf + b * 2 * n;
    const float* E2 = D + n;
    // Gershgorin bounds widened by the FP32 rounding of the counts
    const float tn = (float)info[b * 8 + 4];
    float lo = (float)info[b * 8 + 0] - 8.f * FLT_EPSILON * tn * 64.f, hi = (float)info[b * 8 + 1] + 8.f * FLT_EPSILON * tn * 64.f;
    const float pivmin = fmaxf(1e-30f, (float)info[b * 8 + 3]);
    for (int it = 0; it < 64; ++it) {
        const float width = hi - lo;
        if (width <= 2.f * FLT_EPSILON * fmaxf(fabsf(lo), fabsf(hi)) || width <= pivmin) break;
        const float mid = 0.5f * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (sturm_f32(D, E2, (int)n, mid, pivmin) >= j + 1)
            hi = mid;
        else
            lo = mid;
    }
    w[b * iu + j] = 0.5 * ((double)lo + (double)hi);
}

// cluster starts: clus[b*(iu+1) + 0] = count, followed by start indices (ascending), last = iu
__global__ void k_clusters(const double* __restrict__ w, int64_t iu, const double* __restrict__ info, double ortol_rel,
                           int* __restrict__ clus) {
    const int64_t b = blockIdx.x;
    if (threadIdx.x != 0) return;
    const double* W = w + b * iu;
    int* C = clus + b * (iu + 2);
    const double ortol = ortol_rel * info[b * 8 + 2];
    int cnt = 0;
    for (int64_t j = 0; j < iu; ++j) {
        if (j == 0 || W[j] - W[j - 1] > ortol) C[1 + cnt++] = (int)j;
    }
    C[1 + cnt] = (int)iu;
    C[0] = cnt;
}

__device__ inline uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

// One thread per cluster.  Scratch per thread (strided by 'stride' threads): a, b, c, dd (doubles), piv (bytes).
__global__ void k_invit(const double* __restrict__ d, const double* __restrict__ e, int64_t n, int64_t iu,
                        const double* __restrict__ w, const double* __restrict__ info, const int* __restrict__ clus,
                        double* __restrict__ Z /* batch x (n x iu) row-major */, double* __restrict__ scr,
                        unsigned char* __restrict__ pivs, int64_t stride, int* __restrict__ fail) {
    const int64_t b = blockIdx.y;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int* C = clus + b * (iu + 2);
    const int ncl = C[0];
    if (t >= ncl) return;
    const double* D = d + b * n;
    const double* E = e + b * n;
    const double* Wb = w + b * iu;
    double* Zb = Z + b * n * iu;
    const int64_t th = b * stride + t;              // scratch column
    const int64_t S = stride * gridDim.y;           // scratch row pitch
    double* ua = scr;                               // diag of U
    double* ub = scr + n * S;                       // first super-diag of U
    double* uc = scr + 2 * n * S;                   // multipliers
    double* ud = scr + 3 * n * S;                   // second super-diag of U
    const double onenrm = info[b * 8 + 2];
    const int js = C[1 + t], je = C[2 + t];
    double xjm = 0.0;
    for (int j = js; j < je; ++j) {
        double xj = Wb[j];
        if (j > js) {
            double pertol = 10.0 * fabs(kEps * xj);
            if (xj - xjm < pertol) xj = xjm + pertol;
        }
        xjm = xj;
        // ---- dlagtf: T - xj I = P L U
        int64_t in_n = 0;
        {
            const double tl = kEps;
            double a0 = D[0] - xj;
            ua[th] = a0;
            if (n > 1) ub[th] = E[0];
            double scale1 = fabs(a0) + ((n > 1) ? fabs(E[0]) : 0.0);
            for (int64_t k = 0; k < n - 1; ++k) {
                double ak = ua[k * S + th];
                double bk = ub[k * S + th];
                double ck = E[k];
                double ak1 = D[k + 1] - xj;
                double bk1 = (k < n - 2) ? E[k + 1] : 0.0;
                double scale2 = fabs(ck) + fabs(ak1);
                if (k < n - 2) scale2 += fabs(bk1);
                double piv1 = (ak == 0.0) ? 0.0 : fabs(ak) / scale1;
                double piv2;
                unsigned char pv;
                double dk = 0.0;
                if (ck == 0.0) {
                    pv = 0;
                    piv2 = 0.0;
                    scale1 = scale2;
                    uc[k * S + th] = 0.0;
                } else {
                    piv2 = fabs(ck) / scale2;
                    if (piv2 <= piv1) {
                        pv = 0;
                        scale1 = scale2;
                        double m = ck / ak;
                        uc[k * S + th] = m;
                        ak1 = ak1 - m * bk;
                    } else {
                        pv = 1;
                        double mult = ak / ck;
                        ua[k * S + th] = ck;
                        double temp = ak1;
                        ak1 = bk - mult * temp;
                        if (k < n - 2) {
                            dk = bk1;
                            bk1 = -mult * dk;
                        }
                        ub[k * S + th] = temp;
                        uc[k * S + th] = mult;
                    }
                }
                if (k < n - 2) ud[k * S + th] = dk;
                pivs[k * S + th] = pv;
                if (fmax(piv1, piv2) <= tl && in_n == 0) in_n = k + 1;
                ua[(k + 1) * S + th] = ak1;
                if (k + 1 < n - 1) ub[(k + 1) * S + th] = bk1;
            }
            if (fabs(ua[(n - 1) * S + th]) <= scale1 * tl && in_n == 0) in_n = n;
        }
        // dlagts tolerance for job = -1
        double tol = fabs(ua[th]);
        if (n > 1) tol = fmax(tol, fmax(fabs(ua[S + th]), fabs(ub[th])));
        for (int64_t k = 2; k < n; ++k)
            tol = fmax(tol, fmax(fabs(ua[k * S + th]), fmax(fabs(ub[(k - 1) * S + th]), fabs(ud[(k - 2) * S + th]))));
        tol *= kEps;
        if (tol == 0.0) tol = kEps;
        // ---- starting vector in Z(:, j)
        uint64_t seed = mix64(((uint64_t)b << 40) ^ ((uint64_t)j * 0x9e3779b97f4a7c15ULL) ^ 0x1234567ULL);
        for (int64_t i = 0; i < n; ++i) {
            seed = mix64(seed + 0x9e3779b97f4a7c15ULL);
            Zb[i * iu + j] = (double)(seed >> 11) * (2.0 / 9007199254740992.0) - 1.0;
        }
        const int maxits = 5, extra = 2;
        const double dtpcrt = sqrt(0.1 / (double)n);
        int nrmchk = 0, its = 0;
        bool ok = false;
        while (its < maxits) {
            ++its;
            // scale: scl = n * onenrm * max(eps, |u_nn|) / ||b||_inf
            double bmax = 0.0;
            for (int64_t i = 0; i < n; ++i) bmax = fmax(bmax, fabs(Zb[i * iu + j]));
            double scl = (double)n * onenrm * fmax(kEps, fabs(ua[(n - 1) * S + th])) / bmax;
            // forward: apply P and L
            double yprev = Zb[j] * scl;
            Zb[j] = yprev;
            for (int64_t k = 1; k < n; ++k) {
                double yk = Zb[k * iu + j] * scl;
                const double m = uc[(k - 1) * S + th];
                if (pivs[(k - 1) * S + th] == 0) {
                    yk = yk - m * yprev;
                } else {
                    double temp = yprev;
                    Zb[(k - 1) * iu + j] = yk;
                    yprev = yk;
                    yk = temp - m * yk;
                }
                Zb[k * iu + j] = yk;
                yprev = yk;
            }
            // backward with perturbation of tiny pivots
            double y1 = 0.0, y2 = 0.0;  // y(k+1), y(k+2)
            for (int64_t k = n - 1; k >= 0; --k) {
                double temp = Zb[k * iu + j];
                if (k <= n - 3)
                    temp = temp - ub[k * S + th] * y1 - ud[k * S + th] * y2;
                else if (k == n - 2)
                    temp = temp - ub[k * S + th] * y1;
                double ak = ua[k * S + th];
                double pert = copysign(tol, ak);
                for (int guard = 0; guard < 2048; ++guard) {
                    double absak = fabs(ak);
                    if (absak < 1.0) {
                        if (absak < kSafmin) {
                            if (absak == 0.0 || fabs(temp) * kSafmin > absak) {
                                ak += pert;
                                pert *= 2.0;
                                continue;
                            }
                            temp *= 1.0 / kSafmin;
                            ak *= 1.0 / kSafmin;
                        } else if (fabs(temp) > absak * (1.0 / kSafmin)) {
                            ak += pert;
                            pert *= 2.0;
                            continue;
                        }
                    }
                    break;
                }
                double yk = temp / ak;
                Zb[k * iu + j] = yk;
                y2 = y1;
                y1 = yk;
            }
            // modified Gram-Schmidt against earlier cluster members
            for (int q = js; q < j; ++q) {
                double dot = 0.0;
                for (int64_t i = 0; i < n; ++i) dot += Zb[i * iu + j] * Zb[i * iu + q];
                for (int64_t i = 0; i < n; ++i) Zb[i * iu + j] -= dot * Zb[i * iu + q];
            }
            double nrm = 0.0;
            for (int64_t i = 0; i < n; ++i) nrm = fmax(nrm, fabs(Zb[i * iu + j]));
            if (nrm < dtpcrt) continue;
            ++nrmchk;
            if (nrmchk < extra + 1) continue;
            ok = true;
            break;
        }
        if (!ok) atomicAdd(fail + b, 1);
        // normalise (2-norm), largest component positive
        double s2 = 0.0, big = 0.0;
        int64_t jmax = 0;
        for (int64_t i = 0; i < n; ++i) {
            double v = Zb[i * iu + j];
            s2 += v * v;
            if (fabs(v) > big) {
                big = fabs(v);
                jmax = i;
            }
        }
        double scl = 1.0 / sqrt(s2);
        if (Zb[jmax * iu + j] < 0.0) scl = -scl;
        for (int64_t i = 0; i < n; ++i) Zb[i * iu + j] *= scl;
        (void)in_n;
    }
}

// X (n x iu complex, column-major) = Z (row-major real)
__global__ void k_z_to_x(const double* __restrict__ Z, int64_t n, int64_t iu, double2* __restrict__ X, int64_t ldx,
                         int64_t strideX) {
    const int64_t b = blockIdx.z;
    const int64_t i = blockIdx.x * 32 + threadIdx.x;
    const int64_t j0 = blockIdx.y * 32;
    __shared__ double tile[32][33];
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        int64_t ii = blockIdx.x * 32 + r, jj = j0 + threadIdx.x;
        tile[r][threadIdx.x] = (ii < n && jj < iu) ? Z[b * n * iu + ii * iu + jj] : 0.0;
    }
    __syncthreads();
    for (int c = threadIdx.y; c < 32; c += blockDim.y) {
        int64_t jj = j0 + c;
        if (i < n && jj < iu) X[b * strideX + i + jj * ldx] = make_double2(tile[threadIdx.x][c], 0.0);
    }
}

// ---------------------------------------------------------------- back-transformation (FP64)
// Compact-WY blocks of BT64 reflectors; the two long-K products (the Gram matrix V^H V and
// W = V^H X) are split over K so that their few output tiles still fill the GPU.
constexpr int BT64 = 64;
constexpr int64_t BT64_CTA_TARGET = 2 * 152;

// upper bounds of the K splits (they size the workspace): enough CTAs for the GPU, no split
// shorter than 256 rows
inline void bt64_split_caps(int64_t n, int64_t iu, int64_t batch, int64_t& ksg, int64_t& ksw) {
    const int64_t kmax = std::max<int64_t>(1, (n + 255) / 256);
    ksg = std::min<int64_t>(std::min<int64_t>(32, (BT64_CTA_TARGET + batch - 1) / batch), kmax);
    const int64_t wt = (iu + ZG_BN - 1) / ZG_BN * batch;
    ksw = std::min<int64_t>(std::min<int64_t>(16, (BT64_CTA_TARGET + wt - 1) / wt), kmax);
}

struct BtV {  // V(r, l) of block j0: reflector j0+l, rows >= j0+1 (r relative to j0+1)
    const double2* A;
    int64_t lda, strideA, n, j0, nbk;
    __device__ double2 at(int64_t rr, int64_t l) const {
        const int64_t r = j0 + 1 + rr, j = j0 + l;
        if (l >= nbk || r >= n || r < j + 1) return make_double2(0.0, 0.0);
        if (r == j + 1) return make_double2(1.0, 0.0);
        return A[blockIdx.z * strideA + r + j * lda];
    }
};
struct BtGramA {  // a(l, k) = conj(V(k, l))
    BtV v;
    __device__ double2 operator()(int64_t l, int64_t k) const { return cconj(v.at(k, l)); }
};
struct BtGramB {  // b(i, k) = V(k, i)
    BtV v;
    __device__ double2 operator()(int64_t i, int64_t k) const { return v.at(k, i); }
};
struct BtStoreSmall {  // G(l, i) or W(l, c) stored column-major with leading dim ld
    double2* G;
    int64_t ld, stride;
    __device__ void operator()(int64_t i, int64_t j, double2 c) const { G[blockIdx.z * stride + i + j * ld] = c; }
};
struct BtXk {  // b(c, k) = X(j0+1+k, c)
    const double2* X;
    int64_t ldx, strideX, n, j0, iu;
    __device__ double2 operator()(int64_t c, int64_t k) const {
        const int64_t r = j0 + 1 + k;
        if (c >= iu || r >= n) return make_double2(0.0, 0.0);
        return X[blockIdx.z * strideX + r + c * ldx];
    }
};
struct BtTW_A {  // a(l, q) = T(l, q) upper triangular, BT64 x BT64 column-major
    const double2* T;
    int64_t nbk, stride;
    __device__ double2 operator()(int64_t l, int64_t q) const {
        if (l >= nbk || q >= nbk || q < l) return make_double2(0.0, 0.0);
        return T[blockIdx.z * stride + l + q * BT64];
    }
};
struct BtTW_B {  // b(c, q) = W(q, c), W column-major with leading dimension BT64
    const double2* W;
    int64_t nbk, iu, stride;
    __device__ double2 operator()(int64_t c, int64_t q) const {
        if (q >= nbk || c >= iu) return make_double2(0.0, 0.0);
        return W[blockIdx.z * stride + q + c * BT64];
    }
};
struct BtTW_Bsum {  // b(c, q) = W(q, c) summed over ks K-split partials (partial s at (s * batch + b))
    const double2* W;
    int64_t nbk, iu, ks, batch;
    __device__ double2 operator()(int64_t c, int64_t q) const {
        if (q >= nbk || c >= iu) return make_double2(0.0, 0.0);
        const double2* p = W + blockIdx.z * BT64 * iu + q + c * BT64;
        double2 acc = p[0];
        for (int64_t s = 1; s < ks; ++s) acc = cadd(acc, p[s * batch * BT64 * iu]);
        return acc;
    }
};
struct BtStoreSplit {  // partial s of batch item b at P + (s * batch + b) * stride, leading dimension BT64
    double2* P;
    int64_t stride, batch;
    __device__ void operator()(int64_t s, int64_t i, int64_t j, double2 c) const {
        P[(s * batch + blockIdx.z) * stride + i + j * BT64] = c;
    }
};
struct BtVa {  // a(rr, l) = V(rr, l)
    BtV v;
    __device__ double2 operator()(int64_t rr, int64_t l) const { return v.at(rr, l); }
};
struct BtXUpd {
    double2* X;
    int64_t ldx, strideX, j0;
    __device__ void operator()(int64_t rr, int64_t c, double2 val) const {
        double2* x = X + blockIdx.z * strideX + (j0 + 1 + rr) + c * ldx;
        *x = csub(*x, val);
    }
};

// zlarft (forward, columnwise) from the Gram matrix G = V^H V given as ks K-split partials
// (partial s of batch item b at G + (s * batch + b) BT64^2):
// T(0:i, i) = T(0:i, 0:i) (-tau_i G(0:i, i)), T(i, i) = tau_i.  blockDim.x = BT64, thread l owns row l.
__global__ void k_larft(const double2* __restrict__ G, int64_t ks, int64_t batch, const double2* __restrict__ tau,
                        int64_t n, int64_t j0, int64_t nbk, double2* __restrict__ T) {
    const int64_t b = blockIdx.x;
    double2* Tb = T + b * BT64 * BT64;
    const double2* tb = tau + b * n;
    __shared__ double2 tmp[BT64];
    const int l = threadIdx.x;
    for (int q = l; q < BT64 * BT64; q += blockDim.x) Tb[q] = make_double2(0.0, 0.0);
    __syncthreads();
    for (int64_t i = 0; i < nbk; ++i) {
        const double2 ti = tb[j0 + i];
        if (l < i) {
            double2 g = make_double2(0.0, 0.0);
            for (int64_t s = 0; s < ks; ++s) g = cadd(g, G[(s * batch + b) * BT64 * BT64 + l + i * BT64]);
            tmp[l] = cmul(cmake(-ti.x, -ti.y), g);
        }
        __syncthreads();
        if (l < i) {
            double2 acc = make_double2(0.0, 0.0);
            for (int64_t q = l; q < i; ++q) acc = cadd(acc, cmul(Tb[l + q * BT64], tmp[q]));
            Tb[l + i * BT64] = acc;
        }
        if (l == 0) Tb[i + i * BT64] = ti;
        __syncthreads();
    }
}

int backtransform_fp64(cudaStream_t st, const double2* A, int64_t lda, int64_t strideA, const double2* tau, int64_t n,
                       double2* X, int64_t ldx, int64_t strideX, int64_t iu, int64_t batch, double2* Gws,
                       double2* Tws, double2* Wws, double2* W2ws) {
    const int64_t nrefl = n - 1;
    const int64_t nblocks = (nrefl + BT64 - 1) / BT64;
    int64_t ksg_cap, ksw_cap;
    bt64_split_caps(n, iu, batch, ksg_cap, ksw_cap);
    for (int64_t blk = nblocks - 1; blk >= 0; --blk) {
        const int64_t j0 = blk * BT64;
        const int64_t nbk = (nrefl - j0 < BT64) ? (nrefl - j0) : BT64;
        const int64_t K = n - j0 - 1;
        BtV v{A, lda, strideA, n, j0, nbk};
        // G = V^H V (nbk x nbk), split over K
        const int64_t ksg = zg_ksplit_count(K, std::min<int64_t>(ksg_cap, (K + 255) / 256));
        FORGE_TRY((zgemm_launch_splitk<double2, KMAJOR, KMAJOR>(st, nbk, nbk, K, batch, ksg, BtGramA{v},
                                                                BtGramB{v}, BtStoreSplit{Gws, BT64 * BT64, batch})));
        k_larft<<<(unsigned)batch, BT64, 0, st>>>(Gws, ksg, batch, tau, n, j0, nbk, Tws);
        FORGE_LAUNCH_CHECK();
        // W = V^H X (nbk x iu), split over K
        const int64_t ksw = zg_ksplit_count(K, std::min<int64_t>(ksw_cap, (K + 255) / 256));
        FORGE_TRY((zgemm_launch_splitk<double2, KMAJOR, KMAJOR>(st, nbk, iu, K, batch, ksw, BtGramA{v},
                                                                BtXk{X, ldx, strideX, n, j0, iu},
                                                                BtStoreSplit{Wws, BT64 * iu, batch})));
        // W2 = T W
        FORGE_TRY((zgemm_launch<double2, KMAJOR, KMAJOR, false>(
            st, nbk, iu, nbk, batch, BtTW_A{Tws, nbk, BT64 * BT64}, BtTW_Bsum{Wws, nbk, iu, ksw, batch},
            BtStoreSmall{W2ws, BT64, BT64 * iu})));
        // X(j0+1:, :) -= V W2
        FORGE_TRY((zgemm_launch<double2, IMAJOR, KMAJOR, false>(st, K, iu, nbk, batch, BtVa{v},
                                                                 BtTW_B{W2ws, nbk, iu, BT64 * iu},
                                                                 BtXUpd{X, ldx, strideX, j0})));
    }
    return 0;
}

// ---------------------------------------------------------------- FP64 eigen-solver driver
int eig_fp64(cudaStream_t st, EigArgs& g) {
    const int64_t n = g.n, iu = g.iu, batch = g.batch;
    TrdArgs<double> a;
    a.A = g.A;
    a.lda = g.lda;
    a.strideA = g.strideA;
    a.n = n;
    a.d = g.d;
    a.e = g.e;
    a.tau = g.tau;
    a.W = g.Wp;
    a.Yrow = g.Yrow;
    a.Ycol = g.Ycol;
    a.ystride = g.ystride;
    a.Spart = g.Spart;
    a.sstride = g.sstride;
    a.part = g.part;
    a.pstride = g.pstride;
    a.scal = g.scal;
    a.cnt = g.cnt;
    FORGE_CUDA(cudaMemsetAsync(g.cnt, 0, sizeof(unsigned) * 4 * batch, st));
    FORGE_TRY(tridiagonalize<double>(st, a, batch));
    FORGE_TRY(tridiag_eigvecs(st, g));
    dim3 gz((unsigned)((n + 31) / 32), (unsigned)((iu + 31) / 32), (unsigned)batch);
    k_z_to_x<<<gz, dim3(32, 8), 0, st>>>(g.Z, n, iu, g.X, g.ldx, g.strideX);
    FORGE_LAUNCH_CHECK();
    prof_begin(ST_BACKTRANSFORM);
    FORGE_TRY(backtransform_fp64(st, g.A, g.lda, g.strideA, g.tau, n, g.X, g.ldx, g.strideX, iu, batch, g.G, g.T,
                                 g.Wb, g.W2b));
    prof_end(ST_BACKTRANSFORM, batch * (double)n * iu * 16.0 * 2.0 + batch * 0.5 * n * (double)n * 16.0,
             batch * 8.0 * (double)n * n * iu);
    return 0;
}

// eigenvalues 1..iu (bisection) and tridiagonal eigenvectors (inverse iteration) into g.X (real)
int tridiag_eigvecs(cudaStream_t st, EigArgs& g) {
    const int64_t n = g.n, iu = g.iu, batch = g.batch;
    k_gersh<<<(unsigned)batch, 256, 0, st>>>(g.d, g.e, n, g.info);
    FORGE_LAUNCH_CHECK();
    dim3 gb((unsigned)((iu + 127) / 128), (unsigned)batch);
    prof_begin(ST_BISECT);
    if (g.bisect_f32) {
        k_tri_to_f32<<<dim3((unsigned)std::min<int64_t>((n + 255) / 256, 64), (unsigned)batch), 256, 0, st>>>(
            g.d, g.e, n, g.tf);
        FORGE_LAUNCH_CHECK();
        k_bisect_f32<<<gb, 128, 0, st>>>(g.tf, n, iu, g.info, g.w);
        FORGE_LAUNCH_CHECK();
    }
    // full FP64 accuracy in both paths: inverse iteration on tight clusters needs it (a 1e-10 ||T||
    // stop made the batched inverse iteration 7x slower on the twisted-bilayer spectra)
    k_bisect<<<gb, 128, 0, st>>>(g.d, g.e, n, iu, g.info, g.w, g.bisect_f32, 0.0);
    FORGE_LAUNCH_CHECK();
    prof_end(ST_BISECT, batch * 16.0 * n, batch * 10.0 * 60.0 * (double)n * iu);
    k_clusters<<<(unsigned)batch, 32, 0, st>>>(g.w, iu, g.info, g.ortol_rel, g.clus);
    FORGE_LAUNCH_CHECK();
    FORGE_CUDA(cudaMemsetAsync(g.fail, 0, sizeof(int) * batch, st));
    dim3 gi((unsigned)((g.scr_stride + 63) / 64), (unsigned)batch);
    prof_begin(ST_INVIT);
    k_invit<<<gi, 64, 0, st>>>(g.d, g.e, n, iu, g.w, g.info, g.clus, g.Z, g.scr, g.pivs, g.scr_stride, g.fail);
    FORGE_LAUNCH_CHECK();
    prof_end(ST_INVIT, batch * 8.0 * (double)n * iu, 0.0);
    return 0;
}

}  // namespace forge

namespace forge {

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
void carve(EigArgs& g, Carve& c) {
    const int64_t n = g.n, iu = g.iu, B = g.batch;
    const int64_t nblk = (n + TRD_TILE - 1) / TRD_TILE;
    const int64_t nrb = (n + 255) / 256;
    g.ystride = nblk * n;
    g.sstride = nrb * 2 * TRD_NB;
    g.pstride = 2 * ((n + 31) / 32) + 2;  // per-CTA partials of trd_col / trd_finish
    g.scr_stride = iu;
    g.d = c.take<double>(B * n);
    g.e = c.take<double>(B * n);
    g.tau = c.take<double2>(B * n);
    g.Wp = c.take<double2>(B * n * TRD_NB);
    g.Yrow = c.take<double2>(B * g.ystride);
    g.Ycol = c.take<double2>(B * g.ystride);
    g.Spart = c.take<double2>(B * g.sstride);
    g.part = c.take<double>(B * g.pstride);
    g.scal = c.take<double>(B * 16);
    g.cnt = c.take<unsigned>(B * 4);
    g.info = c.take<double>(B * 8);
    g.clus = c.take<int>(B * (iu + 2));
    g.Z = c.take<double>(B * n * iu);
    g.scr = c.take<double>(4 * n * iu * B);
    g.pivs = c.take<unsigned char>(n * iu * B);
    g.fail = c.take<int>(B);
    int64_t ksg, ksw;
    bt64_split_caps(n, iu, B, ksg, ksw);
    g.G = c.take<double2>(ksg * B * BT64 * BT64);
    g.T = c.take<double2>(B * BT64 * BT64);
    g.Wb = c.take<double2>(ksw * B * BT64 * iu);
    g.W2b = c.take<double2>(B * BT64 * iu);
    g.tf = c.take<float>(B * 2 * n);
}
}  // namespace

size_t eig_workspace_bytes(int64_t n, int64_t iu, int64_t batch) {
    EigArgs g{};
    g.n = n;
    g.iu = iu;
    g.batch = batch;
    Carve c{nullptr};
    carve(g, c);
    return c.off;
}

void eig_bind_workspace(EigArgs& g, void* base) {
    Carve c{static_cast<char*>(base)};
    carve(g, c);
}

}  // namespace forge
