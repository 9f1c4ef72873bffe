// Uneven-size batch of the eigen-solve: the H(k) of systems with different ndim solved in one
// batched launch sequence (no counterpart in the reference, which builds one system per binary,
// Setup.f90:6-74).  Each H(k) of a system with n_b sites is embedded in an n x n slot
// (n = the largest ndim of the group) as
//     [ H   0     ]
//     [ 0   s I   ],   s = 1 + max_i sum_j |H(i,j)|  (Gershgorin: above every eigenvalue of H)
// The Householder reduction leaves the s I block untouched (its columns need no reflector), the
// tridiagonal splits at n_b, and eigenpairs 1..iu <= n_b of the slot are those of H with zero
// padding rows; iu never reaches the s block.
#include <algorithm>

#include "cvec.cuh"
#include "forge_internal.cuh"

namespace forge {

namespace {

// row sums of |H| over the full Hermitian matrix from its lower triangle (rowsum zeroed first)
__global__ void k_row_abs_sum(const double2* __restrict__ H, int64_t n, double* __restrict__ rowsum) {
    const int64_t total = n * n;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / n, i = e - j * n;
        if (i < j) continue;
        const double2 h = H[e];
        const double a = sqrt(h.x * h.x + h.y * h.y);
        atomicAdd(rowsum + i, a);
        if (i != j) atomicAdd(rowsum + j, a);
    }
}

// sigma = 1 + max_i rowsum(i); one CTA of 256 threads
__global__ void k_gershgorin(const double* __restrict__ rowsum, int64_t n, double* __restrict__ sigma) {
    double m = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, rowsum[i]);
    __shared__ double red[8];
    m = warp_max_d(m);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < 8; ++w) t = fmax(t, red[w]);
        *sigma = t + 1.0;
    }
}

// lower triangle of the n x n slot from the nb x nb lower triangle of src
__global__ void k_pad_lower(const double2* __restrict__ src, int64_t nb, double2* __restrict__ dst, int64_t n,
                            const double* __restrict__ sigma) {
    const int64_t total = n * n;
    const double s = *sigma;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = e / n, i = e - j * n;
        double2 v = make_double2(0.0, 0.0);
        if (i < j)
            v = make_double2(0.0, 0.0);   // the strict upper triangle is not read by the solvers
        else if (i < nb && j < nb)
            v = src[i + j * nb];
        else if (i == j)
            v = make_double2(s, 0.0);
        dst[e] = v;
    }
}

unsigned grid_for(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8); }

}  // namespace

// Embeds the nb x nb lower triangle src into the n x n slot dst (see above); rowsum: nb doubles of
// scratch, sigma: one double of scratch.
int launch_pad_slot(cudaStream_t st, const double2* src, int64_t nb, double2* dst, int64_t n, double* rowsum,
                    double* sigma) {
    FORGE_CUDA(cudaMemsetAsync(rowsum, 0, nb * sizeof(double), st));
    k_row_abs_sum<<<grid_for(nb * nb), 256, 0, st>>>(src, nb, rowsum);
    FORGE_LAUNCH_CHECK();
    k_gershgorin<<<1, 256, 0, st>>>(rowsum, nb, sigma);
    FORGE_LAUNCH_CHECK();
    k_pad_lower<<<grid_for(n * n), 256, 0, st>>>(src, nb, dst, n, sigma);
    FORGE_LAUNCH_CHECK();
    return 0;
}

}  // namespace forge
