// Valley projection (nenforceValley = 1, Main.f90:470-500): the window part of the new density
// matrix is the average of GetFock over the window eigenvectors X and over their valley
// transforms X S(k), S(k) = sign(X^H V(k) X) (ValleyTransform, TightBinding.f90:162-208).
//
// V(k) (ValleyPhase, TightBinding.f90:60-157) couples sites of the same sublattice block of a layer
// at next-nearest-neighbour distance (ftvalley, TightBinding.f90:235-270: i sign(cos 3 phi)/sqrt(27)
// for 0.2 < |r_i - r_j| < 1.2), in the home cell and in the three neighbour cells with the Bloch
// phases exp(-+i k.R_c).  The terms do not depend on k: the host lists them once (row, column,
// coefficient, cell code), and the device applies them with the per-k phases.  Host code here is
// compiled with -ffp-contract=off so the separations round as the Fortran expressions do.
#include <cmath>
#include <vector>

#include "forge_internal.cuh"

namespace forge {

namespace {

// ftvalley of the separation (dx, dy) with the 2 x 2 rotation Rm[row][col]: the sign of
// cos(3 phi), or 0 outside the next-nearest-neighbour shell
int ftvalley_sign(double dx, double dy, const double Rm[2][2]) {
    const double rij = std::sqrt(dx * dx + dy * dy);
    if (!(rij < 1.2 && rij > 0.2)) return 0;
    const double x = Rm[0][0] * dx + Rm[0][1] * dy;
    const double y = Rm[1][0] * dx + Rm[1][1] * dy;
    const double pi = 4.0 * std::atan(1.0);
    double phi;
    if (x > 0) {
        phi = std::atan(y / x);
    } else if (x < 0 && y > 0) {
        phi = std::atan(y / x) + pi;
    } else {
        phi = -pi + std::atan(y / x);
    }
    if (x == 0) phi = y > 0 ? pi / 2.0 : -pi / 2.0;
    return std::signbit(std::cos(3.0 * phi)) ? -1 : 1;
}

// W(:, b, k) = V(k) X_win(:, b, k): one thread per (i, b), blockIdx.y = k
__global__ void k_valley_apply(const double2* __restrict__ X, int64_t N, int64_t iu, int64_t c0, int64_t nb,
                               const int64_t* __restrict__ rowp, const int64_t* __restrict__ col,
                               const double* __restrict__ coef, const int* __restrict__ code,
                               const double2* __restrict__ ph, double2* __restrict__ W) {
    const int64_t k = blockIdx.y;
    const double2* Xk = X + (size_t)k * N * iu + (size_t)c0 * N;
    const double2* pk = ph + k * 7;
    const int64_t total = N * nb;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = e / N, i = e - b * N;
        double2 acc = make_double2(0.0, 0.0);
        for (int64_t t = rowp[i]; t < rowp[i + 1]; ++t) {
            const double2 v = cscale(pk[code[t]], coef[t]);
            acc = cadd(acc, cmul(v, Xk[col[t] + b * N]));
        }
        // the terms are i * coef * phase
        W[(size_t)k * N * nb + e] = make_double2(-acc.y, acc.x);
    }
}

// G(a, b, k) = sum_i conj(X_win(i, a, k)) W(i, b, k): one block per (a + nb b, k)
__global__ void k_valley_gram(const double2* __restrict__ X, int64_t N, int64_t iu, int64_t c0, int64_t nb,
                              const double2* __restrict__ W, double2* __restrict__ G) {
    const int64_t k = blockIdx.y, ab = blockIdx.x;
    const int64_t a = ab % nb, b = ab / nb;
    const double2* xa = X + (size_t)k * N * iu + (size_t)(c0 + a) * N;
    const double2* wb = W + (size_t)k * N * nb + (size_t)b * N;
    double2 acc = make_double2(0.0, 0.0);
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) acc = cadd(acc, cjmul(xa[i], wb[i]));
    __shared__ double2 red[256];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] = cadd(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) G[(size_t)k * nb * nb + ab] = red[0];
}

// Xv(:, b, k) = sum_a X_win(:, a, k) S(a, b, k)
__global__ void k_valley_rotate(const double2* __restrict__ X, int64_t N, int64_t iu, int64_t c0, int64_t nb,
                                const double2* __restrict__ S, double2* __restrict__ Xv) {
    const int64_t k = blockIdx.y;
    const double2* Xk = X + (size_t)k * N * iu + (size_t)c0 * N;
    const double2* Sk = S + (size_t)k * nb * nb;
    const int64_t total = N * nb;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = e / N, i = e - b * N;
        double2 acc = make_double2(0.0, 0.0);
        for (int64_t a = 0; a < nb; ++a) acc = cadd(acc, cmul(Xk[i + a * N], Sk[a + b * nb]));
        Xv[(size_t)k * N * nb + e] = acc;
    }
}

unsigned grid_x(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 4096); }

}  // namespace

int valley_build_terms(const Context& c, const int64_t* RotateLayers, ValleyTerms& t) {
    const int64_t N = c.N, nl = c.s.nlayers, per = N / nl;
    // RotMatrix = reshape([cos, -sin, sin, cos], [2, 2]) of half the twist angle (Main.f90:130-133)
    const double m = (double)c.s.ntheta;
    const double cs = 1.0 - 1.0 / (2.0 * (3.0 * m * m + 3.0 * m + 1.0));
    const double th = 0.5 * std::acos(cs);
    const double R[2][2] = {{std::cos(th), std::sin(th)}, {-std::sin(th), std::cos(th)}};
    const double RT[2][2] = {{R[0][0], R[1][0]}, {R[0][1], R[1][1]}};
    const double inv = 1.0 / std::sqrt(27.0);
    const double* X = c.coords_h.data();  // N x 3, column-major
    std::vector<std::vector<std::pair<int64_t, std::pair<int, int>>>> rows(N);  // (j, (sign, code))
    for (int64_t l = 0; l < nl; ++l) {
        const int64_t rl = RotateLayers[l];
        if (rl != -1 && rl != 1) continue;
        const double(*Rm)[2] = rl == -1 ? RT : R;
        const int64_t blocks[2][2] = {{per * l, per * l + per / 2}, {per * l + per / 2, per * (l + 1)}};
        for (const auto& bl : blocks)
            for (int64_t i = bl[0]; i < bl[1]; ++i)
                for (int64_t j = bl[0]; j < bl[1]; ++j) {
                    const double xi = X[i], yi = X[i + N], xj = X[j], yj = X[j + N];
                    int sg = ftvalley_sign(xi - xj, yi - yj, Rm);
                    if (sg) rows[i].push_back({j, {sg, 0}});
                    for (int cc = 1; cc < 4; ++cc) {
                        const double n1 = (double)c.ucell1[cc], n2 = (double)c.ucell2[cc];
                        // r_j - R_c with exp(-i k.R_c); r_i - R_c with exp(+i k.R_c)
                        sg = ftvalley_sign(xi - ((xj - n1 * c.t1[0]) - n2 * c.t2[0]),
                                           yi - ((yj - n1 * c.t1[1]) - n2 * c.t2[1]), Rm);
                        if (sg) rows[i].push_back({j, {sg, cc}});
                        sg = ftvalley_sign(((xi - n1 * c.t1[0]) - n2 * c.t2[0]) - xj,
                                           ((yi - n1 * c.t1[1]) - n2 * c.t2[1]) - yj, Rm);
                        if (sg) rows[i].push_back({j, {sg, 3 + cc}});
                    }
                }
    }
    t.rowp.assign(N + 1, 0);
    t.col.clear();
    t.coef.clear();
    t.code.clear();
    for (int64_t i = 0; i < N; ++i) {
        for (const auto& e : rows[i]) {
            t.col.push_back(e.first);
            t.coef.push_back(e.second.first * inv);
            t.code.push_back(e.second.second);
        }
        t.rowp[i + 1] = (int64_t)t.col.size();
    }
    return 0;
}

void valley_phases(const Context& c, std::vector<double2>& ph) {
    const int64_t Nk = c.Nk, numk = c.s.numk;
    ph.assign(Nk * 7, make_double2(1.0, 0.0));
    for (int64_t k = 0; k < Nk; ++k) {
        const int64_t ivk1 = c.kcomp[k], ivk2 = c.kcomp[k + Nk];
        const double vk0 = c.kvals[ivk1 + ivk2 * numk], vk1 = c.kvals[ivk1 + ivk2 * numk + numk * numk];
        for (int cc = 1; cc < 4; ++cc) {
            const double n1 = (double)c.ucell1[cc], n2 = (double)c.ucell2[cc];
            const double sx = n1 * c.t1[0] + n2 * c.t2[0], sy = n1 * c.t1[1] + n2 * c.t2[1];
            const double kr = vk0 * sx + vk1 * sy;
            ph[k * 7 + cc] = make_double2(std::cos(kr), -std::sin(kr));
            ph[k * 7 + 3 + cc] = make_double2(std::cos(kr), std::sin(kr));
        }
    }
}

int launch_valley_gram(cudaStream_t st, const double2* X, int64_t N, int64_t iu, int64_t c0, int64_t nb, int64_t Nk,
                       const int64_t* rowp, const int64_t* col, const double* coef, const int* code,
                       const double2* ph, double2* W, double2* G) {
    if (Nk > 65535) {
        set_error(FORGE_ERR_ARG, "valley projection: %lld k points exceed one launch", (long long)Nk);
        return FORGE_ERR_ARG;
    }
    k_valley_apply<<<dim3(grid_x(N * nb), (unsigned)Nk), 256, 0, st>>>(X, N, iu, c0, nb, rowp, col, coef, code, ph, W);
    FORGE_LAUNCH_CHECK();
    k_valley_gram<<<dim3((unsigned)(nb * nb), (unsigned)Nk), 256, 0, st>>>(X, N, iu, c0, nb, W, G);
    FORGE_LAUNCH_CHECK();
    return 0;
}

int launch_valley_rotate(cudaStream_t st, const double2* X, int64_t N, int64_t iu, int64_t c0, int64_t nb, int64_t Nk,
                         const double2* S, double2* Xv) {
    k_valley_rotate<<<dim3(grid_x(N * nb), (unsigned)Nk), 256, 0, st>>>(X, N, iu, c0, nb, S, Xv);
    FORGE_LAUNCH_CHECK();
    return 0;
}

}  // namespace forge
