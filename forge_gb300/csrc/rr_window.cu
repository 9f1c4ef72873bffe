// FP64 Rayleigh-Ritz refinement of the eigenpairs around the Fermi level (mixed precision path).
//
// The mixed eigen-solver's eigenpairs are FP32-accurate: about 2e-6 eV in the eigenvalues at every
// size.  Near the Fermi level of a flat-band system the gaps are meV, so that error turns into a
// large mixing between nearby eigenvectors, which the SCF sees as noise in P.  This step takes
// the nw highest computed eigenvectors X_w of each k (the zdiagRed window nLower..nUpper and the
// bands just below it) and re-solves H(k) in their span in FP64:
//   Y = H X_w,  G = X_w^H Y,  S = X_w^H X_w,  S = L L^H,  L^{-1} G L^{-H} = U diag(theta) U^H,
//   X_w <- X_w L^{-H} U,  w <- theta.
// The FP64 H(k) of the batch is still resident; the three products are FP64 GEMMs on the CUDA
// cores (8 N^2 nw FLOP per k for Y) and the nw x nw problem is solved on the host.
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "cvec.cuh"
#include "eig.cuh"
#include "zgemm_engine.cuh"

namespace forge {

constexpr int RR_MAX = 32;

// --------------------------------------------------------------- nw x nw dense part (host)
namespace {
inline double2 cmk(double r, double i) { return make_double2(r, i); }
inline double2 cad(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }
inline double2 csb(double2 a, double2 b) { return cmk(a.x - b.x, a.y - b.y); }
inline double2 cml(double2 a, double2 b) { return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
inline double2 ccj(double2 a) { return cmk(a.x, -a.y); }
inline double cab2(double2 a) { return a.x * a.x + a.y * a.y; }
}  // namespace

// G, S: n x n Hermitian (column-major).  Outputs: theta (ascending) and M = L^{-H} U (n x n).
// Returns 0, or 1 if S is not positive definite.
int rr_small(int n, const double2* G, const double2* S, double* theta, double2* M) {
    std::vector<double2> L((size_t)n * n, cmk(0, 0)), A((size_t)n * n), C((size_t)n * n), V((size_t)n * n);
    auto at = [n](std::vector<double2>& X, int i, int j) -> double2& { return X[(size_t)i + (size_t)j * n]; };
    // Cholesky S = L L^H (lower)
    for (int j = 0; j < n; ++j) {
        double d = S[(size_t)j + (size_t)j * n].x;
        for (int k = 0; k < j; ++k) d -= cab2(at(L, j, k));
        if (!(d > 0.0)) return 1;
        const double ljj = std::sqrt(d);
        at(L, j, j) = cmk(ljj, 0);
        for (int i = j + 1; i < n; ++i) {
            double2 s = S[(size_t)i + (size_t)j * n];
            for (int k = 0; k < j; ++k) s = csb(s, cml(at(L, i, k), ccj(at(L, j, k))));
            at(L, i, j) = cmk(s.x / ljj, s.y / ljj);
        }
    }
    // C = L^{-1} G (forward substitution on every column)
    for (int c = 0; c < n; ++c)
        for (int i = 0; i < n; ++i) {
            double2 s = G[(size_t)i + (size_t)c * n];
            for (int k = 0; k < i; ++k) s = csb(s, cml(at(L, i, k), at(C, k, c)));
            const double lii = at(L, i, i).x;
            at(C, i, c) = cmk(s.x / lii, s.y / lii);
        }
    // A = L^{-1} C^H = (L^{-1} G L^{-H})^H; Hermitian up to rounding: keep its lower part mirrored
    for (int c = 0; c < n; ++c)
        for (int i = 0; i < n; ++i) {
            double2 s = ccj(at(C, c, i));
            for (int k = 0; k < i; ++k) s = csb(s, cml(at(L, i, k), at(A, k, c)));
            const double lii = at(L, i, i).x;
            at(A, i, c) = cmk(s.x / lii, s.y / lii);
        }
    for (int j = 0; j < n; ++j) {
        at(A, j, j).y = 0.0;
        for (int i = j + 1; i < n; ++i) {
            const double2 m = cmk(0.5 * (at(A, i, j).x + at(A, j, i).x), 0.5 * (at(A, i, j).y - at(A, j, i).y));
            at(A, i, j) = m;
            at(A, j, i) = ccj(m);
        }
    }
    // cyclic Jacobi with exact 2 x 2 unitary rotations
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) at(V, i, j) = cmk(i == j ? 1.0 : 0.0, 0.0);
    double fro = 0.0;
    for (auto& x : A) fro += cab2(x);
    fro = std::sqrt(fro);
    for (int sweep = 0; sweep < 30; ++sweep) {
        double off = 0.0;
        for (int j = 0; j < n; ++j)
            for (int i = j + 1; i < n; ++i) off += cab2(at(A, i, j));
        if (std::sqrt(off) <= 1e-16 * fro) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double2 c = at(A, p, q);   // A(p, q)
                const double r = std::sqrt(cab2(c));
                if (r == 0.0) continue;
                const double a = at(A, p, p).x, b = at(A, q, q).x;
                const double dl = 0.5 * (b - a), hyp = std::hypot(dl, r);
                // lambda1 - a for the smaller eigenvalue, without cancellation
                const double la = dl > 0.0 ? -r * r / (dl + hyp) : dl - hyp;
                // eigenvector of the smaller eigenvalue: (c, lambda1 - a) normalised; the other is
                // its orthogonal complement (-conj(v1_q), conj(v1_p))
                const double nrm = std::sqrt(r * r + la * la);
                const double2 u0 = cmk(c.x / nrm, c.y / nrm), u1 = cmk(la / nrm, 0.0);
                const double2 w0 = cmk(-u1.x, u1.y), w1 = ccj(u0);
                // A <- W^H A W on rows / columns p, q; V <- V W, W = [[u0, w0], [u1, w1]]
                for (int k = 0; k < n; ++k) {
                    const double2 akp = at(A, k, p), akq = at(A, k, q);
                    at(A, k, p) = cad(cml(akp, u0), cml(akq, u1));
                    at(A, k, q) = cad(cml(akp, w0), cml(akq, w1));
                }
                for (int k = 0; k < n; ++k) {
                    const double2 apk = at(A, p, k), aqk = at(A, q, k);
                    at(A, p, k) = cad(cml(ccj(u0), apk), cml(ccj(u1), aqk));
                    at(A, q, k) = cad(cml(ccj(w0), apk), cml(ccj(w1), aqk));
                }
                at(A, p, q) = cmk(0, 0);
                at(A, q, p) = cmk(0, 0);
                at(A, p, p).y = 0.0;
                at(A, q, q).y = 0.0;
                for (int k = 0; k < n; ++k) {
                    const double2 vkp = at(V, k, p), vkq = at(V, k, q);
                    at(V, k, p) = cad(cml(vkp, u0), cml(vkq, u1));
                    at(V, k, q) = cad(cml(vkp, w0), cml(vkq, w1));
                }
            }
    }
    // ascending order
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return at(A, x, x).x < at(A, y, y).x; });
    // M = L^{-H} V (back substitution with L^H, column by column, in sorted order)
    for (int jj = 0; jj < n; ++jj) {
        const int j = ord[jj];
        theta[jj] = at(A, j, j).x;
        for (int i = n - 1; i >= 0; --i) {
            double2 s = at(V, i, j);
            for (int k = i + 1; k < n; ++k) s = csb(s, cml(ccj(at(L, k, i)), M[(size_t)k + (size_t)jj * n]));
            const double lii = at(L, i, i).x;
            M[(size_t)i + (size_t)jj * n] = cmk(s.x / lii, s.y / lii);
        }
    }
    return 0;
}

// --------------------------------------------------------------- device products
struct RrHermA {  // a(i, k) = H(i, k) from the lower triangle of H (batch item blockIdx.z)
    const double2* H;
    int64_t n, strideH;
    __device__ double2 operator()(int64_t i, int64_t k) const {
        if (i >= n || k >= n) return make_double2(0.0, 0.0);
        const double2* h = H + blockIdx.z * strideH;
        if (i > k) return h[i + k * n];
        if (i == k) return make_double2(h[i + i * n].x, 0.0);
        const double2 u = h[k + i * n];
        return make_double2(u.x, -u.y);
    }
};
struct RrXcol {  // b(j, k) = X(k, c0 + j)
    const double2* X;
    int64_t ldx, strideX, n, c0, nw;
    __device__ double2 operator()(int64_t j, int64_t k) const {
        if (j >= nw || k >= n) return make_double2(0.0, 0.0);
        return X[blockIdx.z * strideX + k + (c0 + j) * ldx];
    }
};
struct RrXcolConj {  // a(i, k) = conj(X(k, c0 + i))
    RrXcol x;
    __device__ double2 operator()(int64_t i, int64_t k) const { return vconj(x(i, k)); }
};
struct RrYcol {  // b(j, k) = Y(k, j)
    const double2* Y;
    int64_t n, nw;
    __device__ double2 operator()(int64_t j, int64_t k) const {
        if (j >= nw || k >= n) return make_double2(0.0, 0.0);
        return Y[blockIdx.z * n * nw + k + j * n];
    }
};
struct RrStoreY {
    double2* Y;
    int64_t n, nw;
    __device__ void operator()(int64_t i, int64_t j, double2 c) const { Y[blockIdx.z * n * nw + i + j * n] = c; }
};
struct RrStoreSmall {  // K-split partial s of batch item b: P + ((s * batch + b) * nw * nw)
    double2* P;
    int64_t nw, batch;
    __device__ void operator()(int64_t s, int64_t i, int64_t j, double2 c) const {
        P[(s * batch + blockIdx.z) * nw * nw + i + j * nw] = c;
    }
};
struct RrMB {  // b(j, k) = M(k, j) of batch item blockIdx.z
    const double2* M;
    int64_t nw;
    __device__ double2 operator()(int64_t j, int64_t k) const {
        if (j >= nw || k >= nw) return make_double2(0.0, 0.0);
        return M[blockIdx.z * nw * nw + k + j * nw];
    }
};
struct RrXcolA {  // a(i, k) = X(i, c0 + k)
    RrXcol x;
    __device__ double2 operator()(int64_t i, int64_t k) const {
        if (k >= x.nw || i >= x.n) return make_double2(0.0, 0.0);
        return x.X[blockIdx.z * x.strideX + i + (x.c0 + k) * x.ldx];
    }
};

__global__ void k_rr_copyback(const double2* __restrict__ T, double2* __restrict__ X, int64_t n, int64_t nw,
                              int64_t c0, int64_t ldx, int64_t strideX) {
    const int64_t b = blockIdx.y;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n * nw; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q % n, j = q / n;
        X[b * strideX + i + (c0 + j) * ldx] = T[b * n * nw + q];
    }
}

size_t rr_window_workspace_bytes(int64_t n, int64_t batch) {
    // Y and the refined vectors (n x RR_MAX each), K-split partials of G and S, M
    return (2 * (size_t)n * RR_MAX + 2 * 16 * (size_t)RR_MAX * RR_MAX + RR_MAX * RR_MAX) * batch * sizeof(double2) +
           256;
}

// Refines columns [c0, c0 + nw) of X and w for every matrix of the batch (H: the FP64 lower triangles).
int rr_window(cudaStream_t st, const double2* H, int64_t strideH, double2* X, int64_t ldx, int64_t strideX, double* w,
              int64_t iu, int64_t n, int64_t c0, int64_t nw, int64_t batch, void* ws) {
    if (nw <= 0) return 0;
    if (nw > RR_MAX || c0 < 0 || c0 + nw > iu) {
        set_error(FORGE_ERR_ARG, "rr_window: window [%lld, %lld) outside 1..%lld or wider than %d", (long long)c0,
                  (long long)(c0 + nw), (long long)iu, RR_MAX);
        return FORGE_ERR_ARG;
    }
    double2* Y = static_cast<double2*>(ws);
    double2* T = Y + (size_t)n * nw * batch;
    double2* Gp = T + (size_t)n * nw * batch;
    const int64_t kmax = 16;
    double2* Sp = Gp + (size_t)kmax * nw * nw * batch;
    double2* Md = Sp + (size_t)kmax * nw * nw * batch;
    prof_begin(ST_REFINE);
    RrXcol xc{X, ldx, strideX, n, c0, nw};
    FORGE_TRY((zgemm_launch<double2, IMAJOR, KMAJOR, false>(st, n, nw, n, batch, RrHermA{H, n, strideH}, xc,
                                                            RrStoreY{Y, n, nw})));
    const int64_t ks = zg_ksplit_count(n, std::min<int64_t>(kmax, (n + 511) / 512));
    FORGE_TRY((zgemm_launch_splitk<double2, KMAJOR, KMAJOR>(st, nw, nw, n, batch, ks, RrXcolConj{xc},
                                                            RrYcol{Y, n, nw}, RrStoreSmall{Gp, nw, batch})));
    FORGE_TRY((zgemm_launch_splitk<double2, KMAJOR, KMAJOR>(st, nw, nw, n, batch, ks, RrXcolConj{xc}, xc,
                                                            RrStoreSmall{Sp, nw, batch})));
    const size_t nn = (size_t)nw * nw;
    std::vector<double2> gp(ks * batch * nn), sp(ks * batch * nn), M(batch * nn);
    std::vector<double> wh(batch * iu);
    FORGE_CUDA(cudaMemcpyAsync(gp.data(), Gp, gp.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
    FORGE_CUDA(cudaMemcpyAsync(sp.data(), Sp, sp.size() * sizeof(double2), cudaMemcpyDeviceToHost, st));
    FORGE_CUDA(cudaMemcpyAsync(wh.data(), w, wh.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    FORGE_CUDA(cudaStreamSynchronize(st));
    // the small problems of the batch in parallel host threads
    auto solve_one = [&](int64_t b) {
        std::vector<double2> G(nn, make_double2(0, 0)), S(nn, make_double2(0, 0));
        for (int64_t s = 0; s < ks; ++s)
            for (size_t q = 0; q < nn; ++q) {
                const double2 g = gp[(s * batch + b) * nn + q], v = sp[(s * batch + b) * nn + q];
                G[q] = make_double2(G[q].x + g.x, G[q].y + g.y);
                S[q] = make_double2(S[q].x + v.x, S[q].y + v.y);
            }
        std::vector<double> th(nw);
        if (rr_small((int)nw, G.data(), S.data(), th.data(), M.data() + b * nn)) {
            // S not positive definite (cannot happen for orthonormal-to-FP32 columns): keep the input
            for (size_t q = 0; q < nn; ++q) M[b * nn + q] = make_double2((q % (nw + 1)) == 0 ? 1.0 : 0.0, 0.0);
            return;
        }
        for (int64_t j = 0; j < nw; ++j) wh[b * iu + c0 + j] = th[j];
    };
    {
        const int64_t nt = std::max<int64_t>(1, std::min<int64_t>(batch, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (int64_t t = 0; t < nt; ++t)
            pool.emplace_back([&, t]() {
                for (int64_t b = t; b < batch; b += nt) solve_one(b);
            });
        for (auto& th : pool) th.join();
    }
    FORGE_CUDA(cudaMemcpyAsync(Md, M.data(), M.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
    FORGE_CUDA(cudaMemcpyAsync(w, wh.data(), wh.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    // X_w <- X_w M (into T, then back into X)
    FORGE_TRY((zgemm_launch<double2, IMAJOR, KMAJOR, false>(st, n, nw, nw, batch, RrXcolA{xc}, RrMB{Md, nw},
                                                            RrStoreY{T, n, nw})));
    k_rr_copyback<<<dim3(256, (unsigned)batch), 256, 0, st>>>(T, X, n, nw, c0, ldx, strideX);
    FORGE_LAUNCH_CHECK();
    // the host vectors above must outlive the asynchronous copies
    FORGE_CUDA(cudaStreamSynchronize(st));
    prof_end(ST_REFINE, batch * (double)n * n * 16.0, batch * 8.0 * (double)n * n * nw);
    return 0;
}

}  // namespace forge

using namespace forge;

// Host-only check of the nw x nw Rayleigh-Ritz solve (no GPU needed): theta and M for given G, S.
extern "C" int forge_selftest_rr_small(int64_t n, const double* G, const double* S, double* theta, double* M) {
    if (n < 1 || n > RR_MAX || !G || !S || !theta || !M) {
        set_error(FORGE_ERR_ARG, "selftest_rr_small: bad arguments");
        return FORGE_ERR_ARG;
    }
    return rr_small((int)n, reinterpret_cast<const double2*>(G), reinterpret_cast<const double2*>(S), theta,
                    reinterpret_cast<double2*>(M));
}
