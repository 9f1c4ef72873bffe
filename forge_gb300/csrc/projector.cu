// K5 / K6: density-matrix projectors (FP64 engine).
//
// Bulk (Solve, HartreeFock.f90:456-473): for each k, C_k = conj(Psi) Psi^T over the
// fully occupied bands 1..nLower-1, accumulated with the integer Bloch phase into
// the four cells:  bulk_c += exp(-2 pi i (ivk1 n1 + ivk2 n1 + ivk2 n2)/numk) C_k.
// C_k is Hermitian, so only its lower triangle is formed and the epilogue writes
// (i,j) and (j,i).  One launch per k keeps the accumulation order fixed.
//
// Window (GetFock, HartreeFock.f90:487-560): sorted states 1..nOcc with weight 1 or
// zdeg; the weight can be complex (reference mode of zdeg), so the full N x N
// product is formed, one GEMM per cell (grid z = cell).
#include "proj.cuh"
#include "zgemm_engine.cuh"

namespace forge {

struct ProjA {  // a(i, n) = conj(X(i, n))
    const double2* X;
    int64_t ldx, N, K;
    __device__ double2 operator()(int64_t i, int64_t n) const {
        if (i >= N || n >= K) return make_double2(0.0, 0.0);
        return cconj(X[i + n * ldx]);
    }
};
struct ProjB {  // b(j, n) = X(j, n)
    const double2* X;
    int64_t ldx, N, K;
    __device__ double2 operator()(int64_t j, int64_t n) const {
        if (j >= N || n >= K) return make_double2(0.0, 0.0);
        return X[j + n * ldx];
    }
};
struct ProjEpi {
    double2* P;  // 4 x N x N
    int64_t N;
    double2 ph[4];
    __device__ void operator()(int64_t i, int64_t j, double2 v) const {
        const size_t NN = (size_t)N * N;
        const size_t oij = i + (size_t)j * N, oji = j + (size_t)i * N;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            double2 t = cmul(ph[c], v);
            P[c * NN + oij] = cadd(P[c * NN + oij], t);
            if (i != j) P[c * NN + oji] = cadd(P[c * NN + oji], cmul(ph[c], cconj(v)));
        }
    }
};

int bulk_projector_fp64(cudaStream_t st, const double2* X, int64_t ldx, int64_t N, int64_t K, const double2 ph[4],
                        double2* P) {
    ProjEpi ep{P, N, {ph[0], ph[1], ph[2], ph[3]}};
    prof_begin(ST_PROJECTOR);
    int rc = zgemm_launch<double2, IMAJOR, IMAJOR, true>(st, N, N, K, 1, ProjA{X, ldx, N, K}, ProjB{X, ldx, N, K}, ep);
    prof_end(ST_PROJECTOR, (double)N * K * 16.0 + 4.0 * 2.0 * N * N * 16.0, 4.0 * (double)N * N * K);
    return rc;
}

struct WinA {  // a(i, s) = conj(psi_s(i)) * w_s * ph_c(k_s),  c = blockIdx.z
    const WinState* st;
    const double2* X;
    int64_t ldx, strideX, N, K;
    __device__ double2 operator()(int64_t i, int64_t s) const {
        if (i >= N || s >= K) return make_double2(0.0, 0.0);
        const WinState w = st[s];
        const double2 x = X[w.k * strideX + i + w.col * ldx];
        return cmul(cconj(x), w.wph[blockIdx.z]);
    }
};
struct WinB {  // b(j, s) = psi_s(j)
    const WinState* st;
    const double2* X;
    int64_t ldx, strideX, N, K;
    __device__ double2 operator()(int64_t j, int64_t s) const {
        if (j >= N || s >= K) return make_double2(0.0, 0.0);
        const WinState w = st[s];
        return X[w.k * strideX + j + w.col * ldx];
    }
};
struct WinEpi {
    double2* P;
    int64_t N;
    __device__ void operator()(int64_t i, int64_t j, double2 v) const {
        double2* p = P + (size_t)blockIdx.z * N * N + i + (size_t)j * N;
        *p = cadd(*p, v);
    }
};

int window_projector_fp64(cudaStream_t st, const WinState* states, int64_t nstates, const double2* X, int64_t ldx,
                          int64_t strideX, int64_t N, double2* P) {
    if (nstates <= 0) return 0;
    prof_begin(ST_WINDOW);
    int rc = zgemm_launch<double2, IMAJOR, IMAJOR, false>(st, N, N, nstates, 4,
                                                          WinA{states, X, ldx, strideX, N, nstates},
                                                          WinB{states, X, ldx, strideX, N, nstates},
                                                          WinEpi{P, N});
    prof_end(ST_WINDOW, (double)N * nstates * 16.0 + 4.0 * 2.0 * N * N * 16.0, 4.0 * 8.0 * (double)N * N * nstates);
    return rc;
}

}  // namespace forge
