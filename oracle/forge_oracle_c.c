/*
 * CPU oracle, C part (TEST INFRASTRUCTURE ONLY).
 *
 * A second, independent restatement of the reference's pair functions and
 * O(N^2) loops, used by oracle/forge_oracle.py to build pair tables and the
 * long-range Hartree kernel at sizes numpy is too slow for, and timed as the
 * CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs
 * may load it.  Parity with the reference is unpinned (no reference tests,
 * no Fortran compiler); see forge_oracle.py's header.
 *
 * Compiled with -ffp-contract=off so that a*b+c is never fused, matching the
 * reference's default (non-FMA) x86-64 code generation.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

typedef struct {
    double a0, r0, d0, tz, xi;
    int64_t nlayers, nscreen;
} fo_model;

/* TightBinding.f90:216-230 */
static double fo_ft(const fo_model* p, const double* ri, double xj, double yj, double zj) {
    double dx = ri[0] - xj, dy = ri[1] - yj, dz = ri[2] - zj;
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    if (!(r > 0.001)) return 0.0;
    double cs = dz / r;
    return -2.7 * exp((p->a0 - r) / p->r0) * (1 - cs * cs) + 0.48 * exp((p->d0 - r) / p->r0) * cs * cs;
}

/* HartreeFock.f90:1232-1274 */
static double fo_fv(const fo_model* p, const double* ri, double xj, double yj, double zj) {
    const double xi = p->xi;
    double dx = ri[0] - xj, dy = ri[1] - yj, dz = ri[2] - zj;
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    double r2 = sqrt(dx * dx + dy * dy);
    double v = 0.0;
    if (p->nscreen == 2) {
        if (r > 0.01) {
            if ((r2 < xi) || (r2 < 2 * p->nlayers * p->tz)) {
                double rho2 = (xj - ri[0]) * (xj - ri[0]) + (yj - ri[1]) * (yj - ri[1]);
                for (int n = -20; n <= 20; ++n) {
                    double sg = (n & 1) ? -1.0 : 1.0;
                    double zz = zj - (n * xi + ri[2] * sg);
                    v = v + sg / sqrt(rho2 + zz * zz);
                }
            } else {
                v = 2.0 * sqrt(2.0) / sqrt(r2 / xi) * exp(-M_PI * r2 / xi) / xi;
            }
        }
    } else if (p->nscreen == 1) {
        if (r > 0.01) {
            double zz = ri[2] + zj + xi;
            v = 1.0 / r - 1.0 / sqrt(dx * dx + dy * dy + zz * zz);
        }
    }
    return v;
}

/*
 * Pair tables for cells c = 0..nnc-1 with shifts sh[2c], sh[2c+1] = n1 t1 + n2 t2 (components
 * evaluated as in the reference: x - n1*t1x - n2*t2x).  Output layout: table[c][i][j] row-major
 * (i = first site), i.e. tm[(c*N + i)*N + j] = ft(r_i, r_j - R_c).
 */
void fo_pair_tables(int64_t N, const double* coords /* N x 3 row-major */, int64_t nnc, const int64_t* u1,
                    const int64_t* u2, const double* t1, const double* t2, const fo_model* p, double* tm,
                    double* tp, double* vm, double* vp) {
    for (int64_t c = 0; c < nnc; ++c) {
        const double n1 = (double)u1[c], n2 = (double)u2[c];
#pragma omp parallel for schedule(dynamic, 4)
        for (int64_t i = 0; i < N; ++i) {
            const double* ri = coords + 3 * i;
            for (int64_t j = 0; j < N; ++j) {
                const double* rj = coords + 3 * j;
                double xm = rj[0] - n1 * t1[0] - n2 * t2[0];
                double ym = rj[1] - n1 * t1[1] - n2 * t2[1];
                double xp = rj[0] + n1 * t1[0] + n2 * t2[0];
                double yp = rj[1] + n1 * t1[1] + n2 * t2[1];
                size_t o = ((size_t)c * N + i) * N + j;
                tm[o] = fo_ft(p, ri, xm, ym, rj[2]);
                tp[o] = fo_ft(p, ri, xp, yp, rj[2]);
                vm[o] = fo_fv(p, ri, xm, ym, rj[2]);
                vp[o] = fo_fv(p, ri, xp, yp, rj[2]);
            }
        }
    }
}

/* HartreeFock.f90:14-53: LR(n,m) for m >= n, mirrored.  LR row-major N x N (symmetric). */
void fo_long_range(int64_t N, const double* coords, const double* t1, const double* t2, int64_t numC,
                   const fo_model* p, double* LR) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t n = 0; n < N; ++n) {
        const double* rn = coords + 3 * n;
        for (int64_t m = n; m < N; ++m) {
            const double* rm = coords + 3 * m;
            double acc = 0.0;
            for (int64_t n1 = -numC; n1 <= numC; ++n1)
                for (int64_t n2 = -numC; n2 <= numC; ++n2) {
                    if (n1 + n2 <= numC && n1 + n2 >= -numC) {
                        double s[3];
                        s[0] = rn[0] - n1 * t1[0] - n2 * t2[0];
                        s[1] = rn[1] - n1 * t1[1] - n2 * t2[1];
                        s[2] = rn[2];
                        acc = acc + fo_fv(p, s, rm[0], rm[1], rm[2]);
                    }
                }
            LR[n * N + m] = acc;
        }
    }
    for (int64_t n = 0; n < N; ++n)
        for (int64_t m = n + 1; m < N; ++m) LR[m * N + n] = LR[n * N + m];
}

/* Rank-1 projector accumulation as the reference performs it (HartreeFock.f90:456-464 via
 * LapackRoutines.f90:168-183): C += conj(psi) psi^T for each of nb columns of Z (column-major N x ld).
 * Interleaved complex doubles.  This is the CPU timing path, not a fast algorithm. */
void fo_rank1_projector(int64_t N, int64_t nb, const double* Z, int64_t ldz, double* C) {
    for (int64_t b = 0; b < nb; ++b) {
        const double* psi = Z + 2 * b * ldz;
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < N; ++j) {
            double pjr = psi[2 * j], pji = psi[2 * j + 1];
            double* col = C + 2 * j * N;
            for (int64_t i = 0; i < N; ++i) {
                /* conj(psi_i) * psi_j */
                double ar = psi[2 * i], ai = -psi[2 * i + 1];
                col[2 * i] += ar * pjr - ai * pji;
                col[2 * i + 1] += ar * pji + ai * pjr;
            }
        }
    }
}

/* HamiltonianHartreeFock (HartreeFock.f90:57-127) for one k with ft / fv evaluated per pair as the
 * reference does (no tables): H lower triangle, column-major N x N interleaved complex.
 * P: zFock (N x N x 4, column-major interleaved).  cell c = 1..3 shifts R_c = n1 t1 + n2 t2. */
void fo_hamiltonian_k(int64_t N, const double* coords /* N x 3 row-major */, const int64_t* u1, const int64_t* u2,
                      const double* t1, const double* t2, const fo_model* p, double alpha, const double* V,
                      const double* P, const double* vk, double* H) {
    const size_t NN = (size_t)N * N;
    double ph[4][2];
    for (int c = 1; c < 4; ++c) {
        double rx = u1[c] * t1[0] + u2[c] * t2[0], ry = u1[c] * t1[1] + u2[c] * t2[1];
        double th = vk[0] * rx + vk[1] * ry;
        ph[c][0] = cos(th);
        ph[c][1] = -sin(th); /* exp(-i k.R) */
    }
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t j = 0; j < N; ++j) {
        const double* rj = coords + 3 * j;
        for (int64_t i = j; i < N; ++i) {
            const double* ri = coords + 3 * i;
            const size_t oij = i + j * (size_t)N, oji = j + i * (size_t)N;
            double hr = (i == j) ? V[i] : 0.0, hi = 0.0;
            double v0 = fo_fv(p, ri, rj[0], rj[1], rj[2]);
            hr += -alpha * v0 * P[2 * oij];
            hi += alpha * v0 * P[2 * oij + 1];
            hr += fo_ft(p, ri, rj[0], rj[1], rj[2]);
            for (int c = 1; c < 4; ++c) {
                const double n1 = (double)u1[c], n2 = (double)u2[c];
                const double er = ph[c][0], ei = ph[c][1];
                double xm = rj[0] - n1 * t1[0] - n2 * t2[0], ym = rj[1] - n1 * t1[1] - n2 * t2[1];
                double xp = rj[0] + n1 * t1[0] + n2 * t2[0], yp = rj[1] + n1 * t1[1] + n2 * t2[1];
                double tm = fo_ft(p, ri, xm, ym, rj[2]), tp = fo_ft(p, ri, xp, yp, rj[2]);
                hr += tm * er + tp * er;
                hi += tm * ei - tp * ei;
                double vm = fo_fv(p, ri, xm, ym, rj[2]);
                double rs[3] = {rj[0], rj[1], rj[2]};
                double vt = fo_fv(p, rs, ri[0] - n1 * t1[0] - n2 * t2[0], ri[1] - n1 * t1[1] - n2 * t2[1], ri[2]);
                const double* pc = P + 2 * (c * NN);
                double ar = pc[2 * oij], ai = -pc[2 * oij + 1]; /* conj(P_c(i,j)) */
                hr += -alpha * vm * (ar * er - ai * ei);
                hi += -alpha * vm * (ar * ei + ai * er);
                double br = pc[2 * oji], bi = pc[2 * oji + 1]; /* P_c(j,i) e^{+ikR} */
                hr += -alpha * vt * (br * er + bi * ei);
                hi += -alpha * vt * (bi * er - br * ei);
            }
            H[2 * oij] = hr;
            H[2 * oij + 1] = hi;
        }
    }
}

/* GetKineticEnergy + GetFockEnergy (HartreeFock.f90:1012-1145) with ft / fv per pair. out[0]=kinetic, out[1]=fock */
void fo_energies_kf(int64_t N, const double* coords, const int64_t* u1, const int64_t* u2, const double* t1,
                    const double* t2, const fo_model* p, const double* P, double* out) {
    const size_t NN = (size_t)N * N;
    double ek = 0.0, ef = 0.0;
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : ek, ef)
    for (int64_t i = 0; i < N; ++i) {
        const double* ri = coords + 3 * i;
        for (int64_t j = 0; j < N; ++j) {
            const double* rj = coords + 3 * j;
            const size_t oij = i + j * (size_t)N, oji = j + i * (size_t)N;
            ek += fo_ft(p, ri, rj[0], rj[1], rj[2]) * P[2 * oij];
            ef += -0.5 * fo_fv(p, ri, rj[0], rj[1], rj[2]) * (P[2 * oij] * P[2 * oij] + P[2 * oij + 1] * P[2 * oij + 1]);
            for (int c = 1; c < 4; ++c) {
                const double n1 = (double)u1[c], n2 = (double)u2[c];
                double xm = rj[0] - n1 * t1[0] - n2 * t2[0], ym = rj[1] - n1 * t1[1] - n2 * t2[1];
                double xp = rj[0] + n1 * t1[0] + n2 * t2[0], yp = rj[1] + n1 * t1[1] + n2 * t2[1];
                const double* pc = P + 2 * (c * NN);
                ek += fo_ft(p, ri, xm, ym, rj[2]) * pc[2 * oij] + fo_ft(p, ri, xp, yp, rj[2]) * pc[2 * oji];
                ef += -0.5 * fo_fv(p, ri, xm, ym, rj[2]) * (pc[2 * oij] * pc[2 * oij] + pc[2 * oij + 1] * pc[2 * oij + 1]);
                ef += -0.5 * fo_fv(p, ri, xp, yp, rj[2]) * (pc[2 * oji] * pc[2 * oji] + pc[2 * oji + 1] * pc[2 * oji + 1]);
            }
        }
    }
    out[0] = ek;
    out[1] = ef;
}
