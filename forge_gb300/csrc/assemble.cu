// K3: batched Hartree-Fock Hamiltonian assembly (HamiltonianHartreeFock,
// HartreeFock.f90:57-127) for a range of k points in one launch.
//
// Each element (i >= j) of the lower triangle is the same affine function of the
// k-dependent phases e_c(k) = exp(-i k.R_c) for every k:
//   H_k(i,j) = A0 + sum_c [ B_c e_c(k) + C_c conj(e_c(k)) ]
//   A0  = V_i delta_ij + bias_i delta_ij + t0 - alpha v0 conj(P0(i,j))
//   B_c = tm_c - alpha vm_c conj(P_c(i,j))           (HartreeFock.f90:91, 108)
//   C_c = tp_c - alpha vt_c P_c(j,i)                 (HartreeFock.f90:95, 110)
// so the tables and P(R) are read once per element and all H(k) are written from
// registers: algorithmic bytes = tables + P once, plus 16 B per written element.
// P_c(j,i) is read through a shared-memory transpose so every global access
// coalesces along i (column-major).
#include "forge_internal.cuh"

namespace forge {

constexpr int ASM_T = 32;       // tile edge
constexpr int ASM_KCHUNK = 256; // phases staged in shared memory per chunk

struct AsmArgs {
    const double* tt;   // 7 tables
    const double* tv;   // 10 tables
    const double2* P;   // 4 x N x N
    const double* V;    // N
    const double2* kph; // Nk x 3 : exp(-i theta_c(k)), c = 1..3
    const double* coords;
    const double* kvec; // Nk x 2 (vk per flat k), used when fphase != 0
    double alpha, Delta, fphase;
    int64_t N, nlayers, k0, nk;
    double2* H;         // nk x N x N
};

__global__ void __launch_bounds__(256) k_assemble(AsmArgs a) {
    const int64_t bi = blockIdx.x, bj = blockIdx.y;
    if (bi < bj) return;
    const int64_t N = a.N;
    const size_t NN = (size_t)N * N;
    const int64_t i = bi * ASM_T + threadIdx.x;
    __shared__ double2 pt[ASM_T][ASM_T + 1];
    __shared__ double2 ph[ASM_KCHUNK][3];
    double2 A0[4], B[3][4], C[3][4];
    // R = 0 part and the B_c terms (direct, coalesced along i)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int64_t j = bj * ASM_T + threadIdx.y + 8 * q;
        A0[q] = make_double2(0.0, 0.0);
#pragma unroll
        for (int c = 0; c < 3; ++c) B[c][q] = C[c][q] = make_double2(0.0, 0.0);
        if (i < N && j < N && i >= j) {
            const size_t o = i + (size_t)j * N;
            const double2 p0 = a.P[o];
            const double v0 = a.tv[o];
            A0[q].x = a.tt[o] - a.alpha * v0 * p0.x;
            A0[q].y = a.alpha * v0 * p0.y;  // -alpha v0 conj(p0)
            if (i == j) {
                double bias = 0.0;
                if (a.nlayers > 1) {
                    const int64_t per = N / a.nlayers;
                    const int64_t l = i / per;
                    bias = ((double)l - (double)(a.nlayers - 1) / 2.0) * a.Delta / (double)(a.nlayers - 1);
                }
                A0[q].x += a.V[i] + bias;
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double2 pc = a.P[(size_t)(c + 1) * NN + o];
                const double vm = a.tv[(size_t)(1 + c) * NN + o];
                B[c][q].x = a.tt[(size_t)(1 + c) * NN + o] - a.alpha * vm * pc.x;
                B[c][q].y = a.alpha * vm * pc.y;
                C[c][q].x = a.tt[(size_t)(4 + c) * NN + o];
            }
        }
    }
    // C_c terms need P_c(j, i): stage the transposed tile
    for (int c = 0; c < 3; ++c) {
        __syncthreads();
        for (int r = threadIdx.y; r < ASM_T; r += 8) {
            // element (row = bj*T + tx, col = bi*T + r) of P_c, coalesced along the row index
            const int64_t rr = bj * ASM_T + threadIdx.x, cc = bi * ASM_T + r;
            pt[r][threadIdx.x] = (rr < N && cc < N) ? a.P[(size_t)(c + 1) * NN + rr + (size_t)cc * N]
                                                    : make_double2(0.0, 0.0);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int64_t j = bj * ASM_T + threadIdx.y + 8 * q;
            if (i < N && j < N && i >= j) {
                const size_t o = i + (size_t)j * N;
                const double2 pji = pt[threadIdx.x][threadIdx.y + 8 * q];  // P_c(j, i)
                const double vt = a.tv[(size_t)(7 + c) * NN + o];
                C[c][q].x -= a.alpha * vt * pji.x;
                C[c][q].y = -a.alpha * vt * pji.y;
            }
        }
    }
    for (int64_t kc = 0; kc < a.nk; kc += ASM_KCHUNK) {
        const int64_t kn = (a.nk - kc < ASM_KCHUNK) ? (a.nk - kc) : ASM_KCHUNK;
        __syncthreads();
        for (int t = threadIdx.x + threadIdx.y * ASM_T; t < kn * 3; t += 256)
            ph[t / 3][t % 3] = a.kph[(a.k0 + kc) * 3 + t];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int64_t j = bj * ASM_T + threadIdx.y + 8 * q;
            if (!(i < N && j < N && i >= j)) continue;
            const size_t o = i + (size_t)j * N;
            double xr = 0.0, yr = 0.0;
            if (a.fphase != 0.0) {
                xr = a.coords[i] - a.coords[j];
                yr = a.coords[i + N] - a.coords[j + N];
            }
            for (int64_t kk = 0; kk < kn; ++kk) {
                double2 h = A0[q];
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const double2 e = ph[kk][c];
                    // B e + C conj(e)
                    h.x += B[c][q].x * e.x - B[c][q].y * e.y + C[c][q].x * e.x + C[c][q].y * e.y;
                    h.y += B[c][q].x * e.y + B[c][q].y * e.x - C[c][q].x * e.y + C[c][q].y * e.x;
                }
                if (a.fphase != 0.0 && i != j) {
                    // zphase = exp(-i vk.(r_i - r_j) fphase) (HartreeFock.f90:79); it is 1 on the diagonal
                    const double* vk = a.kvec + 2 * (a.k0 + kc + kk);
                    const double th = -(vk[0] * xr + vk[1] * yr) * a.fphase;
                    const double cs = cos(th), sn = sin(th);
                    h = make_double2(h.x * cs - h.y * sn, h.x * sn + h.y * cs);
                }
                a.H[(size_t)(kc + kk) * NN + o] = h;
            }
        }
    }
}

int launch_assemble(Context& c, const double* dV, const double2* dP, int64_t k0, int64_t nk, double2* dH) {
    AsmArgs a;
    a.tt = c.tab_t.as<double>();
    a.tv = c.tab_v.as<double>();
    a.P = dP;
    a.V = dV;
    a.kph = c.kphase.as<double2>();
    a.coords = c.coords.as<double>();
    a.kvec = c.kvecs.as<double>();
    a.alpha = c.s.alpha;
    a.Delta = c.s.Delta;
    a.fphase = (double)c.s.fphase;
    a.N = c.N;
    a.nlayers = c.s.nlayers;
    a.k0 = k0;
    a.nk = nk;
    a.H = dH;
    const unsigned nt = (unsigned)((c.N + ASM_T - 1) / ASM_T);
    prof_begin(ST_ASSEMBLE);
    k_assemble<<<dim3(nt, nt), dim3(ASM_T, 8), 0, c.stream>>>(a);
    FORGE_LAUNCH_CHECK();
    // algorithmic bytes: all H(k) lower triangles written + P(R) read once
    const double N = (double)c.N;
    prof_end(ST_ASSEMBLE, nk * N * (N + 1) / 2 * 16.0 + 4.0 * N * N * 16.0, 0.0);
    return 0;
}

}  // namespace forge
