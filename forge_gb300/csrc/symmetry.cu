// Symmetry switches of the SCF loop (Main.f90:513-534), applied to the new density matrix P(R) of
// each iteration (4 cells, N x N complex, column-major):
//   nenforceT   P <- cmplx(real(P), 0)
//   nenforceC2  P(:,:,m) <- (P(:,:,m) + conjg(transpose(P(p, p, m)))) / 2
//   nenforceC2T P(:,:,m) <- (P(:,:,m) + transpose(P(p, p, m))) / 2,   p = nC2pairs
// in that order.  Each C2 average reads a copy of P (the Fortran right-hand side is evaluated
// before the assignment).  HBM bound: one read and one write of P per switch, plus the copy.
#include <algorithm>

#include "cvec.cuh"
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

// Order parameters of P(R = 0): per-CTA partial sums of
//   [0] sum_l (l - (L-1)/2) sum_{i in layer l} (n_i - 1/2)          layer polarisation
//   [1] sum_l (sum_{A block of l} - sum_{B block of l}) (n_i - 1/2)  sublattice polarisation
//   [2] sum_ij |P0(i,j) - P0(c2(j), c2(i))|^2                        C2T breaking (squared)
//   [3] sum_ij |P0(i,j) - P0(c3(i), c3(j))|^2                        C3 breaking (squared)
// c2 / c3: 0-based site maps, or null when the map is incomplete (that norm is not summed).
__global__ void __launch_bounds__(256) k_order_params(const double2* __restrict__ P0, int64_t N, int64_t L,
                                                      const int64_t* __restrict__ c2, const int64_t* __restrict__ c3,
                                                      double* __restrict__ part) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    const int64_t NN = N * N, per = N / L;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < NN; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / N, i = e - j * N;
        const double2 a = P0[e];
        if (i == j) {
            const double dn = a.x - 0.5;
            const int64_t l = i / per;
            acc[0] += ((double)l - 0.5 * (double)(L - 1)) * dn;
            acc[1] += ((i - l * per) < per / 2) ? dn : -dn;
        }
        if (c2) {
            const double2 b = P0[c2[j] + c2[i] * N];
            acc[2] += (a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y);
        }
        if (c3) {
            const double2 b = P0[c3[i] + c3[j] * N];
            acc[3] += (a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y);
        }
    }
    __shared__ double red[8][4];
    for (int t = 0; t < 4; ++t) {
        double v = warp_sum_d(acc[t]);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][t] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0.0;
        for (int w = 0; w < 8; ++w) v += red[w][threadIdx.x];
        part[blockIdx.x * 4 + threadIdx.x] = v;
    }
}

}  // namespace

int launch_order_params(cudaStream_t st, const double2* P0, int64_t N, int64_t L, const int64_t* c2,
                        const int64_t* c3, double* part, int nblocks) {
    k_order_params<<<nblocks, 256, 0, st>>>(P0, N, L, c2, c3, part);
    FORGE_LAUNCH_CHECK();
    return 0;
}

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
