// Host side of the SCF engine: Setup-derived parameters, geometry, and the SCF control
// loop of FORGE's Main.f90, driving the device through the C-ABI of forge_gpu.h.
// Compiled with -ffp-contract=off: the geometry follows the reference's unfused
// double-precision arithmetic so that coordinates and k vectors come out bit for bit
// as a non-FMA evaluation of Geometry.f90 / Main.f90 gives them.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "forge_host.h"

namespace forge {
void set_error(int code, const char* fmt, ...);   // the library's error message (capi.cu)
}

namespace {

const double kA1[2] = {0.5, 0.8660254037844386};   // [0.5, sqrt(3)*0.5]  Setup.f90:71
const double kA2[2] = {-0.5, 0.8660254037844386};  // Setup.f90:72

double pi_ref() { return 4.0 * std::atan(1.0); }  // Setup.f90:74

// the default-real literal 1e-6 of Geometry.f90:154
const double kF32_1em6 = (double)1e-6f;

bool ws_accept(double x1, double x2, int64_t m, double rmax) {
    double r1 = std::fabs(x1 * (3.0 * m + 1) + x2 * (3.0 * m + 2)) + kF32_1em6;
    double r2 = std::fabs(x1 - x2 * (3.0 * m + 1)) + kF32_1em6;
    double r3 = std::fabs(x1 * (3.0 * m + 2) + x2) + kF32_1em6;
    return r1 < rmax && r2 < rmax && r3 < rmax;
}

void rot(const double R[2][2], const double v[2], double out[2]) {
    // matmul(RotMatrix, v) with RotMatrix = reshape([c,-s,s,c],[2,2]) (Main.f90:133)
    double x = R[0][0] * v[0] + R[0][1] * v[1];
    double y = R[1][0] * v[0] + R[1][1] * v[1];
    out[0] = x;
    out[1] = y;
}

// C2 / C3 site maps (Geometry.f90:1140-1223) of N sites in L layers (Coords column-major N x 3).
int site_maps(int64_t N, int64_t L, const double* Coords, int64_t* nC2pairs, int64_t* nC3pairs, int64_t* counts) {
    const int64_t per = N / L;
    int64_t c2cnt = 0, c3cnt = 0;
    if (nC2pairs) {
        for (int64_t i = 0; i < N; ++i) nC2pairs[i] = 0;
        for (int64_t il = 1; il <= L; ++il)
            for (int64_t i = per * (il - 1) + 1; i <= per * (il - 1) + per / 2; ++i)
                for (int64_t j = per * (il - 1) + per / 2 + 1; j <= per * (il - 1) + per; ++j) {
                    double dx = Coords[i - 1] + Coords[j - 1], dy = Coords[i - 1 + N] + Coords[j - 1 + N];
                    if (std::sqrt(dx * dx + dy * dy) < 1e-5) {
                        nC2pairs[i - 1] = j;
                        nC2pairs[j - 1] = i;
                        ++c2cnt;
                    }
                }
    }
    if (nC3pairs) {
        for (int64_t i = 0; i < N; ++i) nC3pairs[i] = 0;
        const double sq = std::sqrt(3.0);
        for (int64_t nl = 1; nl <= L; ++nl) {
            const int64_t base = (nl - 1) * per;
            const int64_t lo[2] = {base + 1, base + per / 2 + 1}, hi[2] = {base + per / 2, base + per};
            for (int h = 0; h < 2; ++h)
                for (int64_t i = lo[h]; i <= hi[h]; ++i) {
                    double x = Coords[i - 1], y = Coords[i - 1 + N];
                    double x3 = -.5 * x - .5 * sq * y, y3 = .5 * sq * x - .5 * y;
                    for (int64_t j = lo[h]; j <= hi[h]; ++j) {
                        double dx = Coords[j - 1] - x3, dy = Coords[j - 1 + N] - y3;
                        if (std::sqrt(dx * dx + dy * dy) < 1e-3) {
                            nC3pairs[i - 1] = j;
                            ++c3cnt;
                        }
                    }
                }
        }
        for (int64_t nl = 1; nl <= L; ++nl) {
            nC3pairs[(nl - 1) * per + per / 2 - 1] = (nl - 1) * per + per / 2;
            nC3pairs[(nl - 1) * per + per - 1] = (nl - 1) * per + per;
            c3cnt += 2;
        }
    }
    if (counts) {
        counts[0] = c2cnt;
        counts[1] = c3cnt;
    }
    return 0;
}

// LatticeRelaxation (Geometry.f90:279-1135) of a bilayer of N sites, Coords column-major N x 3 in
// place.  uqx, uqy: 5 x 5 column-major, uqx[(n-1) + 5 (m-1)] = uqx(n, m).  matched receives the two
// layer-2 quarter counts (matches + 1, ndim/4 each when the re-indexing is a permutation).
int lattice_relaxation(int64_t N, double* Coords, const double g1[2], const double g12[2], const double* uqx,
                       const double* uqy, int64_t matched[2]) {
    const double pi = pi_ref();
    // Gn(1..8) of Geometry.f90:292-299
    const double G[8][2] = {{g1[0], g1[1]},
                            {g12[0], g12[1]},
                            {g12[0] - g1[0], g12[1] - g1[1]},
                            {-g1[0], -g1[1]},
                            {-g12[0], -g12[1]},
                            {-(g12[0] - g1[0]), -(g12[1] - g1[1])},
                            {g1[0], g1[1]},
                            {g12[0], g12[1]}};
    // the 30 Fourier terms in the reference's summation order: nn = 1, 3, 5; n = 2..5; m = 1..n-1
    struct Term {
        double qx, qy, ux, uy;
    };
    std::vector<Term> terms;
    for (int nn = 1; nn <= 5; nn += 2) {
        const double ang = (double)(nn - 1) * pi / 3.0;
        const double ca = std::cos(ang), sa = std::sin(ang);
        for (int n = 2; n <= 5; ++n)
            for (int m = 1; m < n; ++m) {
                const double ux0 = uqx[(n - 1) + 5 * (m - 1)], uy0 = uqy[(n - 1) + 5 * (m - 1)];
                terms.push_back({(double)(n - 1) * G[nn - 1][0] + (double)(m - 1) * G[nn + 1][0],
                                 (double)(n - 1) * G[nn - 1][1] + (double)(m - 1) * G[nn + 1][1],
                                 ca * ux0 - sa * uy0, sa * ux0 + ca * uy0});
            }
    }
    const std::vector<double> nr(Coords, Coords + 3 * N);   // Coordsnr: the unrelaxed sites
    const int64_t half = N / 2;
    // layer 1 moves by delta / 2; layer 2 is its x-mirror (Geometry.f90:1058-1090)
    for (int64_t i = 0; i < half; ++i) {
        const double rx = Coords[i], ry = Coords[i + N];
        double dx = 0.0, dy = 0.0;
        for (const Term& t : terms) {
            const double sv = std::sin(t.qx * rx + t.qy * ry);
            dx = dx - 2.0 * t.ux * sv;
            dy = dy - 2.0 * t.uy * sv;
        }
        Coords[i] = rx + dx / 2.0;
        Coords[i + N] = ry + dy / 2.0;
        Coords[i + half] = -Coords[i];
        Coords[i + half + N] = Coords[i + N];
    }
    // re-index each layer-2 sublattice quarter onto the unrelaxed sites (Geometry.f90:1092-1132)
    std::vector<double> tmp(3 * N, std::numeric_limits<double>::quiet_NaN());
    for (int q = 0; q < 2; ++q) {
        const int64_t lo = q == 0 ? half : 3 * N / 4, hi = q == 0 ? 3 * N / 4 : N;
        int64_t cnt = 0;
        for (int64_t i = lo; i < hi; ++i)
            for (int64_t j = lo; j < hi; ++j) {
                const double ex = Coords[i] - nr[j], ey = Coords[i + N] - nr[j + N];
                if (std::sqrt(ex * ex + ey * ey) < 0.25) {
                    ++cnt;
                    for (int c = 0; c < 3; ++c) tmp[j + c * N] = Coords[i + c * N];
                    break;
                }
            }
        ++cnt;
        tmp[hi - 1] = Coords[hi - 1];
        tmp[hi - 1 + N] = -Coords[hi - 1 + N];
        tmp[hi - 1 + 2 * N] = Coords[hi - 1 + 2 * N];
        matched[q] = cnt;
    }
    for (int c = 0; c < 3; ++c)
        for (int64_t j = half; j < N; ++j) Coords[j + c * N] = tmp[j + c * N];
    return 0;
}

}  // namespace

extern "C" {

int forge_host_setup(forge_setup* s) {
    if (!s || s->nlayers < 1 || s->ntheta < 1 || s->numk < 1) return FORGE_ERR_ARG;
    const int64_t m = s->ntheta;
    s->ndim = s->nlayers * 2 * (m * m + (m + 1) * (m + 1) + (m + 1) * m);  // Setup.f90:10
    s->numb = s->ndim < 20 ? s->ndim : 20;                                  // Setup.f90:23
    const int64_t ncb = s->numb / 2;                                         // Setup.f90:24
    s->nLower = (s->ndim - 2 * s->numb + 2 * ncb) / 2 + 1;                   // Setup.f90:67
    s->nUpper = (s->ndim + 2 * ncb) / 2;                                     // Setup.f90:68
    s->NeutralityPoint = (s->ndim / 2 - s->nLower) + 1;                      // Setup.f90:69
    // Geometry.f90:14-35
    int64_t cnt = 0;
    for (int64_t n1 = -s->numI; n1 <= s->numI; ++n1)
        for (int64_t n2 = -s->numI; n2 <= s->numI; ++n2)
            if (n1 + n2 <= s->numI && n1 + n2 >= -s->numI && (n1 != 0 || n2 != 0)) ++cnt;
    s->numNeighborCells = cnt / 2 + 1;
    s->alpha = 5.853 / s->epsilon * 1.0;   // Setup.f90:58
    s->alphaH = 5.853 / s->epsilon * 1.0;  // Setup.f90:59
    s->a0 = 1.0 / std::sqrt(3.0);          // Setup.f90:62
    s->r0 = 0.184;                         // Setup.f90:63
    s->d0 = 1.35772 / 1.0;                 // Setup.f90:64 (pressure = 1)
    s->tz = 1.35772 / 1.0;                 // Setup.f90:65
    return 0;
}

int forge_host_geometry(const forge_setup* s, const int64_t* RotateLayers, double* Coords, int64_t* nUnitCell_1,
                        int64_t* nUnitCell_2, double* tn, double* g1o, double* g12o, double* MomentaValues,
                        int64_t* nMomentaComponents, int64_t* nMomentaFlattened, int64_t* nC2pairs,
                        int64_t* nC3pairs, int64_t* counts) {
    if (!s || !RotateLayers || !Coords || !nUnitCell_1 || !nUnitCell_2 || !tn || !MomentaValues ||
        !nMomentaComponents)
        return FORGE_ERR_ARG;
    const int64_t N = s->ndim, m = s->ntheta, numk = s->numk, Nk = numk * numk, L = s->nlayers;
    const double pi = pi_ref();
    // OrderNeighborCells (Geometry.f90:40-91) for numI = 1
    if (s->numNeighborCells != 4) return FORGE_ERR_ARG;
    const int64_t u1[4] = {0, -1, -1, 0}, u2[4] = {0, 0, 1, -1};
    for (int q = 0; q < 4; ++q) {
        nUnitCell_1[q] = u1[q];
        nUnitCell_2[q] = u2[q];
    }
    // reciprocal vectors and rotation (Main.f90:126-136)
    const double aMoire = 3.0 * (double)(m * m) + 3.0 * (double)m + 1.0;
    const double f = (4.0 * pi / 3.0) / aMoire;
    double g1[2] = {f * ((double)(3 * m + 1) * kA1[0] + kA2[0]), f * ((double)(3 * m + 1) * kA1[1] + kA2[1])};
    double g12[2] = {f * ((double)(3 * m + 2) * kA2[0] - kA1[0]), f * ((double)(3 * m + 2) * kA2[1] - kA1[1])};
    const double cs = 1.0 - 1.0 / (2.0 * aMoire);
    const double sn = std::sqrt(1.0 - cs * cs);
    const double th = 0.5 * std::acos(cs);
    const double c = std::cos(th), sg = std::sin(th);
    const double R[2][2] = {{c, sg}, {-sg, c}};
    double tmp[2];
    rot(R, g1, tmp);
    g1[0] = tmp[0];
    g1[1] = tmp[1];
    rot(R, g12, tmp);
    g12[0] = tmp[0];
    g12[1] = tmp[1];
    if (g1o) {
        g1o[0] = g1[0];
        g1o[1] = g1[1];
    }
    if (g12o) {
        g12o[0] = g12[0];
        g12o[1] = g12[1];
    }
    // SampleBZ (Geometry.f90:96-127)
    int64_t icount = 0;
    for (int64_t ivk1 = 0; ivk1 < numk; ++ivk1)
        for (int64_t ivk2 = 0; ivk2 < numk; ++ivk2) {
            nMomentaComponents[icount] = ivk1;
            nMomentaComponents[icount + Nk] = ivk2;
            ++icount;
            if (nMomentaFlattened) nMomentaFlattened[ivk1 + ivk2 * numk] = icount;
        }
    for (int64_t ivk2 = 0; ivk2 < numk; ++ivk2)
        for (int64_t ivk1 = 0; ivk1 < numk; ++ivk1) {
            MomentaValues[ivk1 + ivk2 * numk] = ((double)ivk1 * g1[0] + (double)ivk2 * g12[0]) / (double)numk;
            MomentaValues[ivk1 + ivk2 * numk + Nk] = ((double)ivk1 * g1[1] + (double)ivk2 * g12[1]) / (double)numk;
        }
    // moire lattice vectors (Main.f90:142-144)
    double t1[2] = {(double)m * kA1[0] + (double)(m + 1) * kA2[0], (double)m * kA1[1] + (double)(m + 1) * kA2[1]};
    double t2[2] = {(double)(-m - 1) * kA1[0] + (double)(2 * m + 1) * kA2[0],
                    (double)(-m - 1) * kA1[1] + (double)(2 * m + 1) * kA2[1]};
    // WignerSeitzCell (Geometry.f90:132-273)
    const int64_t nrad = 3 * m;
    const double rmax = 3.0 * (double)(m * m) + 3.0 * (double)m + 1.0;
    const double sq3 = std::sqrt(3.0);
    int64_t nind = 0;
    auto put = [&](double x, double y, double z) -> bool {
        if (nind >= N) return false;
        Coords[nind] = x;
        Coords[nind + N] = y;
        Coords[nind + 2 * N] = z;
        ++nind;
        return true;
    };
    for (int64_t nl = 1; nl <= L; ++nl) {
        const double z = ((double)(float)(nl - 1) - (double)(float)(L - 1) / 2.0) * s->tz;
        const int64_t rl = RotateLayers[nl - 1];
        if (rl == -1) {
            for (int64_t n1 = -nrad; n1 <= nrad; ++n1)
                for (int64_t n2 = -nrad; n2 <= nrad; ++n2) {
                    double an1 = n1 + 1.0 / 3.0, an2 = n2 - 2.0 / 3.0;
                    if (ws_accept(an1, an2, m, rmax) &&
                        !put((n1 + 1.0 / 3.0) * kA1[0] + (n2 - 2.0 / 3.0) * kA2[0],
                             (n1 + 1.0 / 3.0) * kA1[1] + (n2 - 2.0 / 3.0) * kA2[1], z))
                        return FORGE_ERR_ARG;
                }
            if (!put((-t2[0] - t1[0]) / 3.0, (-t2[1] - t1[1]) / 3.0, z)) return FORGE_ERR_ARG;
            for (int64_t n1 = -nrad; n1 <= nrad; ++n1)
                for (int64_t n2 = -nrad; n2 <= nrad; ++n2) {
                    double bn1 = n1 + 2.0 / 3.0, bn2 = n2 - 1.0 / 3.0;
                    if (ws_accept(bn1, bn2, m, rmax) &&
                        !put(bn1 * kA1[0] + bn2 * kA2[0], bn1 * kA1[1] + bn2 * kA2[1], z))
                        return FORGE_ERR_ARG;
                }
            if (!put((t2[0] + t1[0]) / 3.0, (t2[1] + t1[1]) / 3.0, z)) return FORGE_ERR_ARG;
        } else if (rl == 1) {
            for (int64_t n1 = -nrad; n1 <= nrad; ++n1)
                for (int64_t n2 = -nrad; n2 <= nrad; ++n2) {
                    double an1 = (n1 + 1.0 / 3.0) * (cs - sn / sq3) - 2 * (n2 - 2.0 / 3.0) * sn / sq3;
                    double an2 = (n2 - 2.0 / 3.0) * (cs + sn / sq3) + 2 * (n1 + 1.0 / 3.0) * sn / sq3;
                    if (ws_accept(an1, an2, m, rmax) &&
                        !put(an1 * kA1[0] + an2 * kA2[0], an1 * kA1[1] + an2 * kA2[1], z))
                        return FORGE_ERR_ARG;
                }
            if (!put((t1[0] + t2[0]) / 3.0, (t1[1] + t2[1]) / 3.0, z)) return FORGE_ERR_ARG;
            for (int64_t n1 = -nrad; n1 <= nrad; ++n1)
                for (int64_t n2 = -nrad; n2 <= nrad; ++n2) {
                    double bn1 = (n1 + 2.0 / 3.0) * (cs - sn / sq3) - 2 * (n2 - 1.0 / 3.0) * sn / sq3;
                    double bn2 = (n2 - 1.0 / 3.0) * (cs + sn / sq3) + 2 * (n1 + 2.0 / 3.0) * sn / sq3;
                    if (ws_accept(bn1, bn2, m, rmax) &&
                        !put(bn1 * kA1[0] + bn2 * kA2[0], bn1 * kA1[1] + bn2 * kA2[1], z))
                        return FORGE_ERR_ARG;
                }
            if (!put((-t1[0] - t2[0]) / 3.0, (-t1[1] - t2[1]) / 3.0, z)) return FORGE_ERR_ARG;
        } else {
            return FORGE_ERR_ARG;
        }
    }
    if (nind != N) return FORGE_ERR_ARG;
    // rotate (x, y) by RotMatrix; z unchanged (Main.f90:148-150)
    for (int64_t n = 0; n < N; ++n) {
        double v[2] = {Coords[n], Coords[n + N]}, o[2];
        rot(R, v, o);
        Coords[n] = o[0];
        Coords[n + N] = o[1];
    }
    rot(R, t1, tmp);
    t1[0] = tmp[0];
    t1[1] = tmp[1];
    rot(R, t2, tmp);
    t2[0] = tmp[0];
    t2[1] = tmp[1];
    tn[0] = t1[0];
    tn[1] = t1[1];
    tn[2] = t2[0];
    tn[3] = t2[1];
    tn[4] = t2[0] - t1[0];
    tn[5] = t2[1] - t1[1];
    return site_maps(N, L, Coords, nC2pairs, nC3pairs, counts);
}

int forge_host_lattice_relaxation(const forge_setup* s, double* Coords, const double* g1, const double* g12,
                                  const double* uqx, const double* uqy, int64_t* matched) {
    if (!s || !Coords || !g1 || !g12 || !uqx || !uqy) {
        forge::set_error(FORGE_ERR_ARG, "lattice_relaxation: null argument");
        return FORGE_ERR_ARG;
    }
    if (s->nlayers != 2 || s->ndim < 8 || s->ndim % 4) {
        forge::set_error(FORGE_ERR_ARG, "lattice_relaxation: bilayers only (nlayers = %lld, ndim = %lld)",
                  (long long)s->nlayers, (long long)s->ndim);
        return FORGE_ERR_ARG;
    }
    int64_t cnt[2] = {0, 0};
    lattice_relaxation(s->ndim, Coords, g1, g12, uqx, uqy, cnt);
    if (matched) {
        matched[0] = cnt[0];
        matched[1] = cnt[1];
    }
    if (cnt[0] != s->ndim / 4 || cnt[1] != s->ndim / 4) {
        forge::set_error(FORGE_ERR_ARG,
                  "lattice_relaxation: ERROR RELAXATION, layer-2 quarters matched %lld and %lld sites, expected %lld "
                  "(unmatched sites are NaN)",
                  (long long)cnt[0], (long long)cnt[1], (long long)(s->ndim / 4));
        return FORGE_ERR_ARG;
    }
    return 0;
}

int forge_host_site_maps(const forge_setup* s, const double* Coords, int64_t* nC2pairs, int64_t* nC3pairs,
                         int64_t* counts) {
    if (!s || !Coords || s->nlayers < 1 || s->ndim % s->nlayers) return FORGE_ERR_ARG;
    return site_maps(s->ndim, s->nlayers, Coords, nC2pairs, nC3pairs, counts);
}

int forge_host_plot_bands(const forge_setup* s, const double* Bands, double FermiEnergy,
                          const int64_t* nMomentaFlattened, const double* g1, const double* g12, const char* path) {
    if (!s || !Bands || !nMomentaFlattened || !g1 || !g12 || !path) return FORGE_ERR_ARG;
    FILE* f = std::fopen(path, "w");
    if (!f) return FORGE_ERR_ARG;
    // PlotBands (TightBinding.f90:275-369): K - Gamma - M - K path through the k-grid points
    const int64_t numk = s->numk, numb = s->numb, p = 0;
    const double vK1x = (g1[0] + g12[0]) / 3.0, vK1y = (g1[1] + g12[1]) / 3.0;
    const double vMx = (g1[0] + g12[0]) / 2.0, vMy = (g1[1] + g12[1]) / 2.0;
    const double aKG = std::sqrt(vK1x * vK1x + vK1y * vK1y);
    const double aGM = std::sqrt((vMx - g12[0]) * (vMx - g12[0]) + (vMy - g12[1]) * (vMy - g12[1]));
    const double aMK = std::sqrt((vK1x - vMx) * (vK1x - vMx) + (vK1y - vMy) * (vK1y - vMy));
    const double aT = 3 * aKG + aGM + aMK;
    auto mod = [](int64_t a, int64_t b) { return ((a % b) + b) % b; };
    auto line = [&](double x, int64_t ivk1, int64_t ivk2) {
        const int64_t k = nMomentaFlattened[ivk1 + ivk2 * numk] - 1;  // 1-based flat index
        std::fprintf(f, "%16.8f   ", x);
        for (int64_t i = 0; i < numb; ++i) std::fprintf(f, "%16.8f   ", Bands[i + k * numb] - FermiEnergy);
        std::fprintf(f, "\n");
    };
    const double n3 = (double)(numk / 3), n6 = (double)(numk / 6), n2 = (double)(numk / 2);
    for (int64_t ivk = 0; ivk <= numk / 3 - 1; ++ivk)
        line(ivk * aKG / n3 / aT, mod(2 * numk / 3 + ivk, numk), mod(2 * numk / 3 - 2 * ivk + p * numk / 2, numk));
    line(aKG / aT, 0, p * numk / 2);
    for (int64_t ivk = 1; ivk <= numk / 3; ++ivk)
        line(aKG / aT + aKG * ivk / n3 / aT, mod(ivk, numk), mod(numk - 2 * ivk + p * numk / 2, numk));
    for (int64_t ivk = 1; ivk <= numk / 6; ++ivk)
        line(2 * aKG / aT + aMK * ivk / n6 / aT, mod(numk / 3 + ivk, numk), mod(numk / 3 + ivk + p * numk / 2, numk));
    for (int64_t ivk = 1; ivk <= numk / 2 - 1; ++ivk)
        line((2 * aKG + aMK) / aT + aGM * ivk / n2 / aT, mod(numk / 2 - ivk, numk),
             mod(numk / 2 + ivk + p * numk / 2, numk));
    for (int64_t ivk = 0; ivk <= numk / 3; ++ivk)
        line((2 * aKG + aMK + aGM) / aT + ivk * aKG / n3 / aT, mod(ivk, numk), mod(ivk + p * numk / 2, numk));
    std::fclose(f);
    return 0;
}

int forge_host_parameters_string_relax(const forge_setup* s, const char* statename, int64_t nrelax, char* buf,
                                       int64_t buflen) {
    if (!s || !buf || buflen < 8 || nrelax < 0 || nrelax > 9) return FORGE_ERR_ARG;
    // Main.f90:180-183
    char dop = s->nfilling < 0.0 ? '-' : '+';
    std::snprintf(buf, (size_t)buflen,
                  "-%.3s-filling%c%3.1f-numS%lld-i%lld-nlayers%lld-relax%lld-eps%.1f-U%4.2f-screen%lld-xi%.1f-delta%.3f"
                  "-numI%lld-numC%lld-numk%lld-dp8.dat",
                  statename ? statename : "SSS", dop, std::fabs(s->nfilling), (long long)s->numS,
                  (long long)s->ntheta, (long long)s->nlayers, (long long)nrelax, s->epsilon, s->U,
                  (long long)s->nscreen, s->xi * 0.246, s->Delta, (long long)s->numI, (long long)s->numC,
                  (long long)s->numk);
    return 0;
}

int forge_host_parameters_string(const forge_setup* s, const char* statename, char* buf, int64_t buflen) {
    return forge_host_parameters_string_relax(s, statename, 0, buf, buflen);
}

// Fock checkpoint (Main.f90:647-672, 202-234): one complex value per fixed-length record
int forge_host_write_fock(const forge_setup* s, const double* zFock, const char* path, int64_t record_bytes) {
    if (!s || !zFock || !path || record_bytes < 16) return FORGE_ERR_ARG;
    const int64_t N = s->ndim, NC = s->numNeighborCells;
    FILE* f = std::fopen(path, "wb");
    if (!f) return FORGE_ERR_ARG;
    std::vector<unsigned char> row((size_t)N * record_bytes, 0);
    const size_t NN = (size_t)N * N;
    auto put = [&](int64_t slot, int64_t i, int64_t j, int64_t m) {
        const double* z = zFock + 2 * (m * NN + (size_t)i + (size_t)j * N);
        std::memcpy(row.data() + slot * record_bytes, z, 16);
    };
    bool ok = true;
    for (int64_t i = 0; i < N && ok; ++i) {  // R = 0: lower triangle, row i, columns 0..i
        for (int64_t j = 0; j <= i; ++j) put(j, i, j, 0);
        ok = std::fwrite(row.data(), (size_t)record_bytes, (size_t)(i + 1), f) == (size_t)(i + 1);
    }
    for (int64_t m = 1; m < NC && ok; ++m)
        for (int64_t i = 0; i < N && ok; ++i) {
            for (int64_t j = 0; j < N; ++j) put(j, i, j, m);
            ok = std::fwrite(row.data(), (size_t)record_bytes, (size_t)N, f) == (size_t)N;
        }
    ok = (std::fclose(f) == 0) && ok;
    return ok ? 0 : FORGE_ERR_ARG;
}

int forge_host_read_fock(const forge_setup* s, double* zFock, const char* path, int64_t record_bytes) {
    if (!s || !zFock || !path || record_bytes < 16) {
        forge::set_error(FORGE_ERR_ARG, "read_fock: null argument or record length below 16 bytes");
        return FORGE_ERR_ARG;
    }
    const int64_t N = s->ndim, NC = s->numNeighborCells;
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        forge::set_error(FORGE_ERR_ARG, "read_fock: cannot open %s", path);
        return FORGE_ERR_ARG;
    }
    // the whole record stream of Main.f90:647-672 and nothing else: a shorter file is a cut-off
    // checkpoint, a longer one was written for another geometry or record length
    const long long expect = ((long long)N * (N + 1) / 2 + (long long)(NC - 1) * N * N) * record_bytes;
    std::fseek(f, 0, SEEK_END);
    const long long have = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (have != expect) {
        std::fclose(f);
        forge::set_error(FORGE_ERR_ARG, "read_fock: %s holds %lld bytes, a checkpoint of ndim = %lld with %lld-byte "
                         "records holds %lld", path, have, (long long)N, (long long)record_bytes, expect);
        return FORGE_ERR_ARG;
    }
    std::vector<unsigned char> row((size_t)N * record_bytes);
    const size_t NN = (size_t)N * N;
    bool ok = true;
    for (int64_t i = 0; i < N && ok; ++i) {
        ok = std::fread(row.data(), (size_t)record_bytes, (size_t)(i + 1), f) == (size_t)(i + 1);
        for (int64_t j = 0; j <= i && ok; ++j) {
            double z[2];
            std::memcpy(z, row.data() + j * record_bytes, 16);
            double* a = zFock + 2 * ((size_t)i + (size_t)j * N);
            a[0] = z[0];
            a[1] = z[1];
            if (j < i) {  // zFock(j, i, 1) = conjg(zinput)
                double* c = zFock + 2 * ((size_t)j + (size_t)i * N);
                c[0] = z[0];
                c[1] = -z[1];
            }
        }
    }
    for (int64_t m = 1; m < NC && ok; ++m)
        for (int64_t i = 0; i < N && ok; ++i) {
            ok = std::fread(row.data(), (size_t)record_bytes, (size_t)N, f) == (size_t)N;
            for (int64_t j = 0; j < N && ok; ++j)
                std::memcpy(zFock + 2 * (m * NN + (size_t)i + (size_t)j * N), row.data() + j * record_bytes, 16);
        }
    std::fclose(f);
    if (!ok) {
        forge::set_error(FORGE_ERR_ARG, "read_fock: short read from %s", path);
        return FORGE_ERR_ARG;
    }
    for (size_t q = 0; q < 2 * NN * (size_t)NC; ++q)
        if (!std::isfinite(zFock[q])) {
            forge::set_error(FORGE_ERR_NUMERIC, "read_fock: non-finite value in %s (element %zu)", path, q / 2);
            return FORGE_ERR_NUMERIC;
        }
    return 0;
}

// SortEnergies_2Spins (HartreeFock.f90:929-1004).  Counters are 1-based as in the reference; the
// run loops test their bound before reading, where the Fortran reads one element past the list
// (the comparison result is discarded there, so the merged list is the same).
int forge_host_sort_energies_2spins(int64_t numk, int64_t numb, const int64_t* W, const double* se,
                                    double* out) {
    if (numk < 1 || numb < 1 || !W || !se || !out) return FORGE_ERR_ARG;
    const int64_t Nk = numk * numk, n = numb * Nk;
    // W(i, sp) is W[(i-1) + 2*(sp-1)]; every front block and merge bound must lie inside the lists
    for (int sp = 0; sp < 2; ++sp)
        if (W[2 * sp] < 1 || W[2 * sp + 1] < W[2 * sp] || W[2 * sp + 1] > numb + 1) return FORGE_ERR_ARG;
    if (W[2] > 1 && (W[0] - 1) * Nk + 1 > n) return FORGE_ERR_ARG;  // the spin-2 front block reads s2(ncount1)
    const double* s1 = se - 1;      // SortedEnergies_1Spin(:, 1), 1-based
    const double* s2 = se + n - 1;  // SortedEnergies_1Spin(:, 2)
    double* oe = out;
    double* os = out + 2 * n;
    int64_t cb = 0, c1 = 1, c2 = 1;
    auto put = [&](double e, int sp) {
        oe[cb] = e;
        os[cb] = (double)sp;
        ++cb;
    };
    for (int64_t q = 0; q < (W[0] - 1) * Nk; ++q) put(s1[c1++], 1);
    // HartreeFock.f90:949 reads the spin-2 list at the spin-1 counter
    for (int64_t q = 0; q < (W[2] - 1) * Nk; ++q) {
        put(s2[c1], 2);
        ++c2;
    }
    const int64_t lim1 = Nk * (W[1] - 1), lim2 = Nk * (W[3] - 1);
    while (c1 <= lim1 && c2 <= lim2) {
        if (s1[c1] <= s2[c2]) {
            put(s1[c1++], 1);
            while (c1 <= n && s1[c1] <= s2[c2]) put(s1[c1++], 1);
            put(s2[c2++], 2);
        } else {
            put(s2[c2++], 2);
            while (c2 <= n && s2[c2] <= s1[c1]) put(s2[c2++], 2);
            put(s1[c1++], 1);
        }
    }
    while (c1 <= n) put(s1[c1++], 1);
    while (c2 <= n) put(s2[c2++], 2);
    return cb == 2 * n ? 0 : FORGE_ERR_ARG;
}

// Main.f90:416-453: window, merge, the common Fermi level and the per-spin occupations.
int forge_host_fermi_2spins(const forge_setup* s, const double* SortedEnergies_1Spin, double* SortedEnergies_2Spins,
                            int64_t* nFermiLevel, double* FermiEnergy, int64_t* nOccStates, int64_t* nPartOccStates,
                            double* DegFactor) {
    if (!s || !SortedEnergies_1Spin || !nFermiLevel || !FermiEnergy || !nOccStates || !nPartOccStates || !DegFactor)
        return FORGE_ERR_ARG;
    const int64_t Nk = s->numk * s->numk, n = s->numb * Nk, NP = s->NeutralityPoint;
    const int64_t W[4] = {NP - 1, NP + 2 + 1, NP - 1, NP + 2 + 1};  // nWindowSort_2Spins, Main.f90:416-419
    std::vector<double> own;
    double* merged = SortedEnergies_2Spins;
    if (!merged) {
        own.resize((size_t)(4 * n));
        merged = own.data();
    }
    int rc = forge_host_sort_energies_2spins(s->numk, s->numb, W, SortedEnergies_1Spin, merged);
    if (rc) return rc;
    // nFermiLevel = numS * nint(Nk*NP + Nk/2*nfilling), Fortran nint rounding half away from zero
    const double x = (double)(Nk * NP) + (double)Nk / 2.0 * s->nfilling;
    const int64_t nF = 2 * (int64_t)(x >= 0 ? std::floor(x + 0.5) : -std::floor(-x + 0.5));
    if (nF < 1 || nF >= 2 * n) return FORGE_ERR_ARG;
    const double ef = (merged[nF - 1] + merged[nF]) / 2.0;
    const double tol = s->EnergyTolerance;
    int64_t nocc[2] = {0, 0}, npart[2] = {0, 0};
    for (int64_t q = 0; q < 2 * n; ++q) {
        const int k = merged[2 * n + q] == 1.0 ? 0 : 1;
        const double e = merged[q];
        if ((e - ef) < -tol) {
            ++nocc[k];
        } else if (std::fabs(e - ef) < tol) {
            ++npart[k];
            ++nocc[k];
        }
    }
    double deg = 0.0;
    if (npart[0] != 0 || npart[1] != 0)
        deg = 1.0 / (double)(npart[0] + npart[1]) * (double)(nF + npart[0] + npart[1] - nocc[0] - nocc[1]);
    *nFermiLevel = nF;
    *FermiEnergy = ef;
    nOccStates[0] = nocc[0];
    nOccStates[1] = nocc[1];
    nPartOccStates[0] = npart[0];
    nPartOccStates[1] = npart[1];
    *DegFactor = deg;
    return 0;
}

int forge_host_run_scf(forge_ctx* ctx, const forge_scf_options* opts, const double* zFock_init,
                       forge_scf_result* result, forge_iter_report* reports) {
    if (!ctx || !opts || !result) return FORGE_ERR_ARG;
    std::memset(result, 0, sizeof(*result));
    FILE* fe = nullptr;
    FILE* fc = nullptr;
    auto close_files = [&]() {
        if (fe) std::fclose(fe);
        if (fc) std::fclose(fc);
    };
    const bool switching = opts->mixed_until > 0 || opts->mixed_switch_tol > 0.0;
    int rc = forge_gpu_set_precision(ctx, switching ? FORGE_PREC_MIXED : FORGE_PREC_FP64);
    if (rc) return rc;
    auto t0 = std::chrono::steady_clock::now();
    double E[4];
    if (zFock_init) {
        if ((rc = forge_gpu_set_state(ctx, zFock_init))) return rc;
        if ((rc = forge_gpu_prepare_state(ctx, E))) return rc;
    } else {
        rc = forge_gpu_plain_guess(ctx, E);
        if (rc < 0) return rc;
    }
    auto t1 = std::chrono::steady_clock::now();
    result->guess_seconds = std::chrono::duration<double>(t1 - t0).count();
    if (opts->output_dir) {
        // output/Energy<parameters>, output/Convergence<parameters> (Main.f90:352-358)
        forge_setup s;
        char params[256];
        if ((rc = forge_gpu_get_setup(ctx, &s))) return rc;
        forge_host_parameters_string(&s, opts->statename, params, sizeof(params));
        std::string d(opts->output_dir);
        if (!d.empty() && d.back() != '/') d += '/';
        fe = std::fopen((d + "Energy" + params).c_str(), "w");
        fc = std::fopen((d + "Convergence" + params).c_str(), "w");
        if (!fe || !fc) {
            close_files();
            return FORGE_ERR_ARG;
        }
    }
    bool mixed = switching;
    int64_t it = 0;
    double res = 1e300;
    // the mixed phase also ends when its residual stalls near the FP32 noise floor: no new best
    // (by a factor 0.8) in three iterations while within 100x the switch tolerance
    double best = 1e300;
    int stall = 0;
    while (it < opts->itmax) {
        ++it;
        if (mixed && ((opts->mixed_until > 0 && it > opts->mixed_until) ||
                      (opts->mixed_switch_tol > 0.0 &&
                       (res < opts->mixed_switch_tol || (stall >= 3 && res < 100.0 * opts->mixed_switch_tol))))) {
            mixed = false;
            if ((rc = forge_gpu_set_precision(ctx, FORGE_PREC_FP64))) {
                close_files();
                return rc;
            }
        }
        forge_iter_report r;
        std::memset(&r, 0, sizeof(r));
        rc = forge_gpu_scf_iteration(ctx, E, &r);
        if (rc < 0) {
            close_files();
            return rc;
        }
        if (reports) reports[it - 1] = r;
        res = r.residual;
        if (res < 0.8 * best) {
            best = res;
            stall = 0;
        } else {
            ++stall;
        }
        if (fc)  // Main.f90:616-623
            std::fprintf(fc, "%5.1f   %9.6f   %5.3f   %24.9f   \n", (double)it, r.DensityConvergence, r.Step,
                         r.TotalEnergyIn - r.TotalEnergy);
        if (fe)  // Main.f90:625-631
            std::fprintf(fe, "%5.1f   %24.9f   %24.9f   %24.9f   %24.9f   %24.9f   \n", (double)it, r.TotalEnergyIn,
                         2.0 * r.KineticEnergyIn, 2.0 * r.FockEnergyIn, r.HartreeEnergyIn, r.HubbardEnergyIn);
        if (fe && opts->nMomentaFlattened && opts->g1 && opts->g12) {
            // output/Bands-nspin1<parameters> (Main.f90:601-610), rewritten every iteration
            forge_setup s;
            char params[256];
            forge_gpu_get_setup(ctx, &s);
            forge_host_parameters_string(&s, opts->statename, params, sizeof(params));
            std::vector<double> bands((size_t)s.numb * s.numk * s.numk);
            if (forge_gpu_get_bands(ctx, bands.data()) == 0) {
                std::string d(opts->output_dir);
                if (!d.empty() && d.back() != '/') d += '/';
                forge_host_plot_bands(&s, bands.data(), r.FermiEnergy, opts->nMomentaFlattened, opts->g1, opts->g12,
                                      (d + "Bands-nspin1" + params).c_str());
            }
        }
        result->TotalEnergy = r.TotalEnergy;
        if (opts->residual_tol > 0.0 && res < opts->residual_tol && !mixed) {
            result->converged = 1;
            break;
        }
    }
    auto t2 = std::chrono::steady_clock::now();
    result->iterations = it;
    result->residual = res;
    for (int t = 0; t < 4; ++t) result->Energies[t] = E[t];
    result->seconds = std::chrono::duration<double>(t2 - t1).count();
    close_files();
    return 0;
}

}  // extern "C"
