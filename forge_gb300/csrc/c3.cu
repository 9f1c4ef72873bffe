// C3-reduced solve (nenforceC3 = 1, HartreeFock.f90:131-398 and 564-881): the k points of the grid
// fall into C3 orbits {k, C3 k, C3^2 k}; H(k) is solved for the first k of each orbit only, and the
// eigenvectors of the other two are the representative's with rows permuted by nC3pairs (twice
// for C3_RelatedMomenta(k,2), once for C3_RelatedMomenta(k,3)) and the corner sites of each layer
// phased.  The projector of the rotated eigenvectors is the reference's rotated projector
// (zFockBulkTemp(nC3pairs, nC3pairs) with the corner phases), so the bulk and window projectors
// run unchanged over all k.  At the three C3-invariant k the reference averages a projector with
// its two images; the two rotated copies of those k sit in extra eigenvector slots Nk.. and enter
// with weight 1/3.
#include <algorithm>
#include <cmath>

#include "forge_internal.cuh"

namespace forge {

namespace {

__global__ void k_c3_rotate(const double2* __restrict__ Xr, const double* __restrict__ wr, int64_t N, int64_t iu,
                            const int64_t* __restrict__ slot_tab, const int64_t* __restrict__ perm,
                            const double2* __restrict__ phase, double2* __restrict__ X, double* __restrict__ w) {
    const int64_t s = blockIdx.y;
    const int64_t r = slot_tab[2 * s], kind = slot_tab[2 * s + 1];
    const int64_t* pm = perm + kind * N;
    const double2* src = Xr + (size_t)r * N * iu;
    double2* dst = X + (size_t)s * N * iu;
    const double2* ph = phase + (size_t)s * N;
    const int64_t total = N * iu;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t col = e / N, i = e - col * N;
        dst[e] = cmul(src[pm[i] + col * N], ph[i]);
    }
    if (blockIdx.x == 0)
        for (int64_t t = threadIdx.x; t < iu; t += blockDim.x) w[s * iu + t] = wr[r * iu + t];
}

}  // namespace

// invariant points as the reference tests them (HartreeFock.f90:219): icount 1, numk/3*(numk+1)+1,
// 2*numk/3*(numk+1)+1, here 0-based
bool c3_invariant(int64_t numk, int64_t k) {
    return k == 0 || k == numk / 3 * (numk + 1) || k == 2 * numk / 3 * (numk + 1);
}

int c3_build_tables(int64_t numk, int64_t N, int64_t nlayers, const int64_t* kcomp, const int64_t* RotateLayers,
                    C3Tables& t) {
    const int64_t Nk = numk * numk;
    if (numk % 3 != 0) {
        set_error(FORGE_ERR_ARG, "C3-reduced solve: numk = %lld is not a multiple of 3", (long long)numk);
        return FORGE_ERR_ARG;
    }
    for (int64_t k = 0; k < Nk; ++k)
        if (kcomp[k] * numk + kcomp[k + Nk] != k) {
            set_error(FORGE_ERR_ARG, "C3-reduced solve: k grid not in SampleBZ order");
            return FORGE_ERR_ARG;
        }
    auto mod = [numk](int64_t v) { return ((v % numk) + numk) % numk; };
    // C3_RelatedMomenta (HartreeFock.f90:151-166), 0-based
    std::vector<int64_t> k2(Nk), k3(Nk);
    for (int64_t k = 0; k < Nk; ++k) {
        const int64_t a = kcomp[k], b = kcomp[k + Nk];
        k2[k] = mod(-a - b) * numk + mod(a);
        k3[k] = mod(b) * numk + mod(-a - b);
    }
    // MomentaMod_C3 (HartreeFock.f90:168-187)
    std::vector<char> incl(Nk, 0);
    t.reps.clear();
    for (int64_t k = 0; k < Nk; ++k)
        if (!incl[k]) {
            t.reps.push_back(k);
            incl[k] = incl[k2[k]] = incl[k3[k]] = 1;
        }
    int64_t ninv = 0;
    for (int64_t k = 0; k < Nk; ++k) ninv += c3_invariant(numk, k) ? 1 : 0;
    t.nslots = Nk + 2 * ninv;
    t.slot_tab.assign(2 * t.nslots, -1);
    t.extra.assign(Nk, -1);
    t.phase.assign((size_t)t.nslots * N, make_double2(1.0, 0.0));
    const double pi = 4.0 * std::atan(1.0);
    const int64_t per = N / nlayers;
    // corner phases of the rotated eigenvectors (HartreeFock.f90:223-235, 249-261, fphase = 0)
    auto set_phase = [&](int64_t slot, int64_t q) {
        const double th = 2.0 * pi * (double)q / (double)numk;
        const double2 em = make_double2(std::cos(th), -std::sin(th)), ep = make_double2(std::cos(th), std::sin(th));
        double2* z = t.phase.data() + (size_t)slot * N;
        for (int64_t l = 0; l < nlayers; ++l) {
            const int64_t ih = per * l + per / 2 - 1, ie = per * (l + 1) - 1;
            if (RotateLayers[l] == -1) {
                z[ih] = em;
                z[ie] = ep;
            } else if (RotateLayers[l] == 1) {
                z[ih] = ep;
                z[ie] = em;
            }
        }
    };
    auto assign = [&](int64_t slot, int64_t r, int64_t kind, int64_t target) {
        if (slot < 0 || slot >= t.nslots || t.slot_tab[2 * slot] != -1) return false;
        t.slot_tab[2 * slot] = r;
        t.slot_tab[2 * slot + 1] = kind;
        const int64_t a = kcomp[target], b = kcomp[target + Nk];
        if (kind == 1) set_phase(slot, b);
        if (kind == 2) set_phase(slot, a + b);
        return true;
    };
    int64_t next_extra = Nk;
    for (int64_t r = 0; r < (int64_t)t.reps.size(); ++r) {
        const int64_t k = t.reps[r];
        bool ok = assign(k, r, 0, k);
        if (!c3_invariant(numk, k)) {
            ok = ok && assign(k2[k], r, 2, k2[k]) && assign(k3[k], r, 1, k3[k]);
        } else {
            t.extra[k] = next_extra;
            ok = ok && assign(next_extra, r, 1, k3[k]) && assign(next_extra + 1, r, 2, k2[k]);
            next_extra += 2;
        }
        if (!ok) {
            set_error(FORGE_ERR_ARG, "C3-reduced solve: the C3 orbits do not partition the k grid");
            return FORGE_ERR_ARG;
        }
    }
    for (int64_t s = 0; s < t.nslots; ++s)
        if (t.slot_tab[2 * s] < 0) {
            set_error(FORGE_ERR_ARG, "C3-reduced solve: k point %lld has no orbit", (long long)s);
            return FORGE_ERR_ARG;
        }
    return 0;
}

int launch_c3_rotate(cudaStream_t st, const double2* Xr, const double* wr, int64_t N, int64_t iu, int64_t nslots,
                     const int64_t* slot_tab, const int64_t* perm, const double2* phase, double2* X, double* w) {
    if (nslots <= 0) return 0;
    if (nslots > 65535) {
        set_error(FORGE_ERR_ARG, "C3-reduced solve: %lld eigenvector slots exceed one launch", (long long)nslots);
        return FORGE_ERR_ARG;
    }
    const int64_t total = N * iu;
    const unsigned gx = (unsigned)std::min<int64_t>((total + 255) / 256, 1024);
    k_c3_rotate<<<dim3(gx, (unsigned)nslots), 256, 0, st>>>(Xr, wr, N, iu, slot_tab, perm, phase, X, w);
    FORGE_LAUNCH_CHECK();
    return 0;
}

}  // namespace forge
