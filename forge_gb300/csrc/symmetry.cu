// Symmetry switches of the SCF loop (Main.f90:513-534), applied to the new density matrix P(R) of
// each iteration (4 cells, N x N complex, column-major):
//   nenforceT   P <- cmplx(real(P), 0)
//   nenforceC2  P(:,:,m) <- (P(:,:,m) + conjg(transpose(P(p, p, m)))) / 2
//   nenforceC2T P(:,:,m) <- (P(:,:,m) + transpose(P(p, p, m))) / 2,   p = nC2pairs
// in that order.  Each C2 average reads a copy of P (the Fortran right-hand side is evaluated
// before the assignment).  HBM bound: one read and one write of P per switch, plus the copy.
#include <algorithm>

#include "forge_internal.cuh"

namespace forge {

namespace {

__global__ void k_sym_real(double2* __restrict__ P, int64_t n) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        P[e].y = 0.0;
}

// dst(i, j, m) = (src(i, j, m) + [conj] src(p(j), p(i), m)) / 2
__global__ void k_sym_pair(const double2* __restrict__ src, double2* __restrict__ dst, const int64_t* __restrict__ perm,
                           int64_t N, int conj_image) {
    const int64_t NN = N * N, n = 4 * NN;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = e / NN, r = e - c * NN;
        const int64_t j = r / N, i = r - j * N;
        const double2 a = src[e];
        double2 b = src[c * NN + perm[j] + perm[i] * N];
        if (conj_image) b.y = -b.y;
        dst[e] = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y + b.y));
    }
}

unsigned grid_for(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16); }

}  // namespace

int launch_symmetrize(cudaStream_t st, double2* P, double2* scratch, const int64_t* perm, int64_t N, bool T, bool C2,
                      bool C2T) {
    const int64_t n = 4 * N * N;
    if (T) {
        k_sym_real<<<grid_for(n), 256, 0, st>>>(P, n);
        FORGE_LAUNCH_CHECK();
    }
    for (int pass = 0; pass < 2; ++pass) {
        if (!(pass == 0 ? C2 : C2T)) continue;
        FORGE_CUDA(cudaMemcpyAsync(scratch, P, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
        k_sym_pair<<<grid_for(n), 256, 0, st>>>(scratch, P, perm, N, pass == 0 ? 1 : 0);
        FORGE_LAUNCH_CHECK();
    }
    return 0;
}

}  // namespace forge
