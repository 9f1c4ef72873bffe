// K1 / K2: pair tables of the hopping ft and the screened Coulomb kernel fv for the
// 1 + 2*3 cell images, and the long-range Hartree kernel LR.
//
// This translation unit is compiled with --fmad=false so that every a*b+c is rounded
// twice like the reference's (non-FMA) code; with IEEE sqrt and division the fv
// tables then match a non-fused CPU evaluation bit for bit, and ft differs only by
// the last-place rounding of exp().
//
// Work per launch (algorithmic): tables = 17 N^2 doubles written; LR = N^2 doubles.
// Both are FP64-pipe bound (41-term image sums with a divide and a sqrt per term).
#include "forge_internal.cuh"

namespace forge {

// TightBinding.f90:216-230
__device__ double dev_ft(const forge_setup& s, double xi, double yi, double zi, double xj, double yj,
                         double zj) {
    double dx = xi - xj, dy = yi - yj, dz = zi - zj;
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    if (!(r > 0.001)) return 0.0;
    double cs = dz / r;
    return -2.7 * exp((s.a0 - r) / s.r0) * (1 - cs * cs) + 0.48 * exp((s.d0 - r) / s.r0) * cs * cs;
}

// HartreeFock.f90:1232-1274 (nscreen = 2: dual gate, 41 images; nscreen = 1: single gate)
__device__ double dev_fv(const forge_setup& s, double xi, double yi, double zi, double xj, double yj,
                         double zj) {
    const double gate = s.xi;
    double dx = xi - xj, dy = yi - yj, dz = zi - zj;
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    double r2 = sqrt(dx * dx + dy * dy);
    double v = 0.0;
    if (s.nscreen == 2) {
        if (r > 0.01) {
            if ((r2 < gate) || (r2 < 2 * s.nlayers * s.tz)) {
                double rho2 = (xj - xi) * (xj - xi) + (yj - yi) * (yj - yi);
#pragma unroll 1
                for (int n = -20; n <= 20; ++n) {
                    double sg = (n & 1) ? -1.0 : 1.0;
                    double zz = zj - (n * gate + zi * sg);
                    v = v + sg / sqrt(rho2 + zz * zz);
                }
            } else {
                v = 2.0 * sqrt(2.0) / sqrt(r2 / gate) * exp(-M_PI * r2 / gate) / gate;
            }
        }
    } else if (s.nscreen == 1) {
        if (r > 0.01) {
            double zz = zi + zj + gate;
            v = 1.0 / r - 1.0 / sqrt(dx * dx + dy * dy + zz * zz);
        }
    }
    return v;
}

struct CellShifts {
    double n1[4], n2[4];  // integer cell indices (as doubles) of nUnitCell_1/2
    double t1x, t1y, t2x, t2y;
};

// tab_t: t0, tm1..3, tp1..3 ; tab_v: v0, vm1..3, vp1..3, vt1..3   (each N x N column-major)
__global__ void k_pair_tables(forge_setup s, int64_t N, const double* __restrict__ coords, CellShifts sh,
                              double* __restrict__ tt, double* __restrict__ tv) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t j = blockIdx.y;
    if (i >= N || j >= N) return;
    const double xi = coords[i], yi = coords[i + N], zi = coords[i + 2 * N];
    const double xj = coords[j], yj = coords[j + N], zj = coords[j + 2 * N];
    const size_t NN = (size_t)N * N, o = i + (size_t)j * N;
    tt[o] = dev_ft(s, xi, yi, zi, xj, yj, zj);
    tv[o] = dev_fv(s, xi, yi, zi, xj, yj, zj);
    for (int c = 1; c < 4; ++c) {
        // [Coords(j,1:2) - n1*t1 - n2*t2, Coords(j,3)]  (HartreeFock.f90:91)
        const double n1 = sh.n1[c], n2 = sh.n2[c];
        double xm = xj - n1 * sh.t1x - n2 * sh.t2x, ym = yj - n1 * sh.t1y - n2 * sh.t2y;
        double xp = xj + n1 * sh.t1x + n2 * sh.t2x, yp = yj + n1 * sh.t1y + n2 * sh.t2y;
        tt[c * NN + o] = dev_ft(s, xi, yi, zi, xm, ym, zj);
        tt[(3 + c) * NN + o] = dev_ft(s, xi, yi, zi, xp, yp, zj);
        tv[c * NN + o] = dev_fv(s, xi, yi, zi, xm, ym, zj);
        tv[(3 + c) * NN + o] = dev_fv(s, xi, yi, zi, xp, yp, zj);
        // fv(Coords(j,:), [Coords(i,1:2) - n1*t1 - n2*t2, Coords(i,3)])  (HartreeFock.f90:110)
        tv[(6 + c) * NN + o] =
            dev_fv(s, xj, yj, zj, xi - n1 * sh.t1x - n2 * sh.t2x, yi - n1 * sh.t1y - n2 * sh.t2y, zi);
    }
}

// HartreeFock.f90:14-53; thread (n, m) with n <= m sums the 37 cells in the reference's order.
__global__ void k_long_range(forge_setup s, int64_t N, const double* __restrict__ coords, double t1x,
                             double t1y, double t2x, double t2y, double* __restrict__ LR) {
    int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t m = blockIdx.y;
    if (n >= N || m >= N || n > m) return;
    const double xn = coords[n], yn = coords[n + N], zn = coords[n + 2 * N];
    const double xm = coords[m], ym = coords[m + N], zm = coords[m + 2 * N];
    const int64_t nC = s.numC;
    double acc = 0.0;
    for (int64_t n1 = -nC; n1 <= nC; ++n1)
        for (int64_t n2 = -nC; n2 <= nC; ++n2) {
            if (n1 + n2 <= nC && n1 + n2 >= -nC) {
                double sx = xn - n1 * t1x - n2 * t2x;
                double sy = yn - n1 * t1y - n2 * t2y;
                acc = acc + dev_fv(s, sx, sy, zn, xm, ym, zm);
            }
        }
    LR[n + (size_t)m * N] = acc;
    LR[m + (size_t)n * N] = acc;
}

int launch_pair_tables(Context& c) {
    const int64_t N = c.N;
    const size_t NN = (size_t)N * N;
    FORGE_TRY(c.tab_t.ensure(7 * NN * sizeof(double)));
    FORGE_TRY(c.tab_v.ensure(10 * NN * sizeof(double)));
    CellShifts sh{};
    for (int q = 0; q < 4; ++q) {
        sh.n1[q] = (double)c.ucell1[q];
        sh.n2[q] = (double)c.ucell2[q];
    }
    sh.t1x = c.t1[0];
    sh.t1y = c.t1[1];
    sh.t2x = c.t2[0];
    sh.t2y = c.t2[1];
    dim3 blk(128), grd((unsigned)((N + 127) / 128), (unsigned)N);
    k_pair_tables<<<grd, blk, 0, c.stream>>>(c.s, N, c.coords.as<double>(), sh, c.tab_t.as<double>(),
                                             c.tab_v.as<double>());
    FORGE_LAUNCH_CHECK();
    c.tables_ready = true;
    return 0;
}

int launch_long_range(Context& c) {
    const int64_t N = c.N;
    FORGE_TRY(c.LR.ensure((size_t)N * N * sizeof(double)));
    dim3 blk(128), grd((unsigned)((N + 127) / 128), (unsigned)N);
    k_long_range<<<grd, blk, 0, c.stream>>>(c.s, N, c.coords.as<double>(), c.t1[0], c.t1[1], c.t2[0], c.t2[1],
                                            c.LR.as<double>());
    FORGE_LAUNCH_CHECK();
    c.lr_ready = true;
    return 0;
}

}  // namespace forge
