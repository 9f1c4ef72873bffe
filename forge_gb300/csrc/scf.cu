// K7 / K8 / K9: the bandwidth-bound SCF kernels.
//
//   k_energy_tables : combined tables for the energy pass, built once:
//                     wk0 = t0 (+ layer bias on the diagonal), wk_c(i,j) = tm_c(i,j) + tp_c(j,i),
//                     wf0 = v0, wf_c(i,j) = vm_c(i,j) + vp_c(j,i)  (GetKineticEnergy /
//                     GetFockEnergy, HartreeFock.f90:1012-1145, with the (j,i) terms relabelled)
//   k_sort_fermi    : SortEnergies_1Spin's heap sort (TightBinding.f90:984-1027) and the
//                     Fermi level / degeneracy bookkeeping of Main.f90:400-412, one CTA
//   k_energy_pass   : one pass over P_in, P_new and the tables giving the linear kinetic
//                     forms and the three quadratic Fock forms <a,a>, <a,b>, <b,b>; E(s) of
//                     the ODA line search is exactly quadratic, so these reproduce the
//                     reference's three energy evaluations (HartreeFock.f90:1148-1227)
//   k_lr_matvec     : LR (dn_a, dn_b) in one pass over LR (Main.f90:577-585)
//   k_oda           : the step choice of OptimalStep and the energies at the step
//   k_mix           : P <- s P_new + (1-s) P, density, max|dn|, potential (Main.f90:558-595)
// All reductions use fixed CTA partitions and a fixed final order (bitwise repeatable).
#include "cvec.cuh"
#include "proj.cuh"

namespace forge {

constexpr int RED_CTAS = 1024;

__global__ void k_energy_tables(const double* __restrict__ tt, const double* __restrict__ tv, int64_t N,
                                int64_t nlayers, double Delta, double* __restrict__ te) {
    // te: wk0, wk1..3, wf0, wf1..3  (8 x N x N)
    const size_t NN = (size_t)N * N;
    __shared__ double tp[32][33], vp[32][33];
    const int64_t i0 = blockIdx.x * 32, j0 = blockIdx.y * 32;
    for (int c = 0; c < 4; ++c) {
        if (c > 0) {
            __syncthreads();
            for (int r = threadIdx.y; r < 32; r += blockDim.y) {
                // (row j0+tx, col i0+r) of tp_c / vp_c, i.e. X(j, i) for i = i0 + r
                int64_t rr = j0 + threadIdx.x, cc = i0 + r;
                bool ok = rr < N && cc < N;
                tp[r][threadIdx.x] = ok ? tt[(3 + c) * NN + rr + cc * N] : 0.0;
                vp[r][threadIdx.x] = ok ? tv[(3 + c) * NN + rr + cc * N] : 0.0;
            }
            __syncthreads();
        }
        for (int q = threadIdx.y; q < 32; q += blockDim.y) {
            int64_t i = i0 + threadIdx.x, j = j0 + q;
            if (i >= N || j >= N) continue;
            size_t o = i + (size_t)j * N;
            double wk, wf;
            if (c == 0) {
                wk = tt[o];
                wf = tv[o];
                if (i == j && nlayers > 1) {
                    int64_t per = N / nlayers, l = i / per;
                    wk += ((double)l - (double)(nlayers - 1) / 2.0) * Delta / (double)(nlayers - 1);
                }
            } else {
                wk = tt[c * NN + o] + tp[threadIdx.x][q];
                wf = tv[c * NN + o] + vp[threadIdx.x][q];
            }
            te[c * NN + o] = wk;
            te[(4 + c) * NN + o] = wf;
        }
    }
}

int build_energy_tables(Context& c, DevBuf& te) {
    const int64_t N = c.N;
    FORGE_TRY(te.ensure(8 * (size_t)N * N * sizeof(double)));
    dim3 g((unsigned)((N + 31) / 32), (unsigned)((N + 31) / 32));
    k_energy_tables<<<g, dim3(32, 8), 0, c.stream>>>(c.tab_t.as<double>(), c.tab_v.as<double>(), N, c.s.nlayers,
                                                     c.s.Delta, te.as<double>());
    FORGE_LAUNCH_CHECK();
    return 0;
}

// ---------------------------------------------------------------- sort + Fermi
struct SortArgs {
    const double* w;        // Nk x iu eigenvalues (flat k order)
    int64_t iu, Nk, numb, nLower, NP, numS;
    double nfilling, tol;
    int64_t degmode;
    const double2* bph;     // Nk x 4 integer Bloch phases
    double* sorted_e;       // numb*Nk
    int64_t* sorted_idx;    // numb*Nk (1-based flat icount)
    WinState* states;       // numb*Nk
    ScfScalars* sc;
};

__global__ void k_sort_fermi(SortArgs a) {
    extern __shared__ double sm[];
    const int64_t n = a.numb * a.Nk;
    double* e = sm;
    double* ix = sm + n;
    for (int64_t ic = threadIdx.x; ic < n; ic += blockDim.x) {
        // SortEnergies_1Spin: icount = (band-1)*Nk + k, energies(icount) = Bands(band, k)
        int64_t band = ic / a.Nk, k = ic - band * a.Nk;
        e[ic] = a.w[k * a.iu + (a.nLower - 1) + band];
        ix[ic] = (double)(ic + 1);
    }
    __syncthreads();
    if (threadIdx.x == 0 && n > 1) {
        // heap sort of rows (e, ix) on e, 1-based as in dsort_lists
        double* E = e - 1;
        double* I = ix - 1;
        int64_t l = n / 2 + 1, ir = n;
        for (;;) {
            double ce, ci;
            if (l > 1) {
                --l;
                ce = E[l];
                ci = I[l];
            } else {
                ce = E[ir];
                ci = I[ir];
                E[ir] = E[1];
                I[ir] = I[1];
                --ir;
                if (ir == 1) {
                    E[1] = ce;
                    I[1] = ci;
                    break;
                }
            }
            int64_t i = l, j = 2 * l;
            while (j <= ir) {
                if (j < ir && E[j] < E[j + 1]) ++j;
                if (ce < E[j]) {
                    E[i] = E[j];
                    I[i] = I[j];
                    i = j;
                    j = 2 * j;
                } else {
                    j = ir + 1;
                }
            }
            E[i] = ce;
            I[i] = ci;
        }
    }
    __syncthreads();
    for (int64_t q = threadIdx.x; q < n; q += blockDim.x) {
        a.sorted_e[q] = e[q];
        a.sorted_idx[q] = (int64_t)llrint(ix[q]);
    }
    __shared__ int64_t s_nocc, s_npart;
    __shared__ double s_ef, s_deg;
    if (threadIdx.x == 0) {
        // Main.f90:400-412 (Fortran nint: half away from zero)
        double x = (double)(a.Nk * a.NP) + (double)a.Nk / 2.0 * a.nfilling;
        int64_t nF = a.numS * (int64_t)((x >= 0) ? floor(x + 0.5) : -floor(-x + 0.5));
        double ef = 0.0;
        if (nF >= 1 && nF < n) ef = (e[nF - 1] + e[nF]) / 2.0;
        int64_t nocc = 0, npart = 0;
        for (int64_t q = 0; q < n; ++q) {
            if ((e[q] - ef) < -a.tol) {
                ++nocc;
            } else if (fabs(e[q] - ef) < a.tol) {
                ++nocc;
                ++npart;
            }
        }
        double deg = 1.0 / (double)npart * (double)(nF + npart - nocc);
        a.sc->EF = ef;
        a.sc->DegFactor = deg;
        a.sc->nF = nF;
        a.sc->nOcc = nocc;
        a.sc->nPart = npart;
        a.sc->nStates = nocc;
        // zdeg = cmplx(DegFactor, dp): real part rounded to default (single) kind, imaginary part dp = 8
        double zr = a.degmode == FORGE_DEG_REFERENCE ? (double)(float)deg : deg;
        double zi = a.degmode == FORGE_DEG_REFERENCE ? 8.0 : 0.0;
        a.sc->zdeg_re = zr;
        a.sc->zdeg_im = zi;
        s_nocc = nocc;
        s_npart = npart;
        s_ef = ef;
        s_deg = deg;
    }
    __syncthreads();
    const double2 zdeg = make_double2(a.sc->zdeg_re, a.sc->zdeg_im);
    for (int64_t q = threadIdx.x; q < s_nocc; q += blockDim.x) {
        int64_t icount = (int64_t)llrint(ix[q]);
        int64_t band = (icount - 1) / a.Nk, k = (icount - 1) - band * a.Nk;
        WinState st;
        st.k = k;
        st.col = (a.nLower - 1) + band;
        double2 wgt = (q < s_nocc - s_npart) ? make_double2(1.0, 0.0) : zdeg;
        for (int c = 0; c < 4; ++c) st.wph[c] = cmul(a.bph[k * 4 + c], wgt);
        a.states[q] = st;
    }
    (void)s_ef;
    (void)s_deg;
}

int launch_sort_fermi(Context& c, const double* w, double nfilling, double* sorted_e, int64_t* sorted_idx,
                      WinState* states, ScfScalars* sc) {
    SortArgs a;
    a.w = w;
    a.iu = c.nUpper;
    a.Nk = c.Nk;
    a.numb = c.numb;
    a.nLower = c.nLower;
    a.NP = c.NP;
    a.numS = 1;
    a.nfilling = nfilling;
    a.tol = c.s.EnergyTolerance;
    a.degmode = c.s.degfactor_mode;
    a.bph = c.bphase.as<double2>();
    a.sorted_e = sorted_e;
    a.sorted_idx = sorted_idx;
    a.states = states;
    a.sc = sc;
    const size_t smem = 2 * sizeof(double) * (size_t)(c.numb * c.Nk);
    if (smem > 200 * 1024) {
        set_error(FORGE_ERR_ARG, "window of %lld states exceeds the on-chip sort", (long long)(c.numb * c.Nk));
        return FORGE_ERR_ARG;
    }
    FORGE_CUDA(cudaFuncSetAttribute(k_sort_fermi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    prof_begin(ST_SORT);
    k_sort_fermi<<<1, 256, smem, c.stream>>>(a);
    FORGE_LAUNCH_CHECK();
    prof_end(ST_SORT, (double)(c.numb * c.Nk) * 32.0, 0.0);
    return 0;
}

// ---------------------------------------------------------------- energy pass
__device__ inline double block_sum(double v, double* sh) {
    v = warp_sum_d(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_sum_d(r);
    }
    return r;
}
__device__ inline double block_max(double v, double* sh) {
    v = warp_max_d(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = (l < (int)(blockDim.x >> 5)) ? sh[l] : 0.0;
        r = warp_max_d(r);
    }
    return r;
}

// partials: RED_CTAS x 8 : Kin_a, Kin_b, Qaa, Qab, Qbb, Mres
__global__ void __launch_bounds__(256) k_energy_pass(const double* __restrict__ te, const double2* __restrict__ Pa,
                                                     const double2* __restrict__ Pb, int64_t N, double alpha,
                                                     double* __restrict__ partials) {
    const size_t NN = (size_t)N * N, total = 4 * NN;
    const size_t chunk = (total + gridDim.x - 1) / gridDim.x;
    const size_t beg = blockIdx.x * chunk, end = (beg + chunk < total) ? beg + chunk : total;
    double ka = 0, kb = 0, qaa = 0, qab = 0, qbb = 0, mres = 0;
    for (size_t q = beg + threadIdx.x; q < end; q += blockDim.x) {
        const size_t c = q / NN, o = q - c * NN;
        const double wk = te[c * NN + o], wf = te[(4 + c) * NN + o];
        const double2 a = Pa[q], b = Pb[q];
        ka += wk * a.x;
        kb += wk * b.x;
        qaa += wf * (a.x * a.x + a.y * a.y);
        qab += wf * (a.x * b.x + a.y * b.y);
        qbb += wf * (b.x * b.x + b.y * b.y);
        const double dx = b.x - a.x, dy = b.y - a.y;
        const double wmag = (c == 0) ? fabs(wf) : 0.5 * fabs(wf);
        mres = fmax(mres, alpha * wmag * sqrt(dx * dx + dy * dy));
    }
    __shared__ double sh[32];
    double r0 = block_sum(ka, sh), r1 = block_sum(kb, sh), r2 = block_sum(qaa, sh), r3 = block_sum(qab, sh),
           r4 = block_sum(qbb, sh), r5 = block_max(mres, sh);
    if (threadIdx.x == 0) {
        double* p = partials + blockIdx.x * 8;
        p[0] = r0;
        p[1] = r1;
        p[2] = r2;
        p[3] = r3;
        p[4] = r4;
        p[5] = r5;
    }
}

__global__ void k_reduce_forms(const double* __restrict__ partials, int nparts, ScfScalars* sc) {
    if (threadIdx.x != 0) return;
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int q = 0; q < nparts; ++q) {
        for (int t = 0; t < 5; ++t) s[t] += partials[q * 8 + t];
        s[5] = fmax(s[5], partials[q * 8 + 5]);
    }
    for (int t = 0; t < 6; ++t) sc->forms[t] = s[t];
}

// y_a = LR dn_a, y_b = LR dn_b ; partial over column chunks: part[chunk][2N]
constexpr int LR_CHUNKS = 32;
__global__ void __launch_bounds__(256) k_lr_matvec(const double* __restrict__ LR, const double* __restrict__ da,
                                                   const double* __restrict__ db, int64_t N,
                                                   double* __restrict__ part) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t cs = (N + LR_CHUNKS - 1) / LR_CHUNKS;
    const int64_t m0 = blockIdx.y * cs, m1 = (m0 + cs < N) ? m0 + cs : N;
    if (n >= N) return;
    double ya = 0.0, yb = 0.0;
    for (int64_t m = m0; m < m1; ++m) {
        const double l = LR[n + (size_t)m * N];
        ya += l * (da[m] - 0.5);
        yb += l * (db[m] - 0.5);
    }
    part[(size_t)blockIdx.y * 2 * N + n] = ya;
    part[(size_t)blockIdx.y * 2 * N + N + n] = yb;
}

// finishes y_a, y_b (into y[0..2N)) and the Hartree / Hubbard forms
__global__ void __launch_bounds__(256) k_lr_finish(const double* __restrict__ part, const double* __restrict__ da,
                                                   const double* __restrict__ db, int64_t N, double* __restrict__ y,
                                                   double* __restrict__ hpart) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double haa = 0, hab = 0, hbb = 0, uaa = 0, uab = 0, ubb = 0;
    if (n < N) {
        double ya = 0.0, yb = 0.0;
        for (int q = 0; q < LR_CHUNKS; ++q) {
            ya += part[(size_t)q * 2 * N + n];
            yb += part[(size_t)q * 2 * N + N + n];
        }
        y[n] = ya;
        y[N + n] = yb;
        const double a = da[n] - 0.5, b = db[n] - 0.5;
        haa = a * ya;
        hab = a * yb;
        hbb = b * yb;
        uaa = a * a;
        uab = a * b;
        ubb = b * b;
    }
    __shared__ double sh[32];
    double r0 = block_sum(haa, sh), r1 = block_sum(hab, sh), r2 = block_sum(hbb, sh), r3 = block_sum(uaa, sh),
           r4 = block_sum(uab, sh), r5 = block_sum(ubb, sh);
    if (threadIdx.x == 0) {
        double* p = hpart + blockIdx.x * 8;
        p[0] = r0;
        p[1] = r1;
        p[2] = r2;
        p[3] = r3;
        p[4] = r4;
        p[5] = r5;
    }
}

__global__ void k_reduce_hforms(const double* __restrict__ hpart, int nparts, ScfScalars* sc) {
    if (threadIdx.x != 0) return;
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int q = 0; q < nparts; ++q)
        for (int t = 0; t < 6; ++t) s[t] += hpart[q * 8 + t];
    for (int t = 0; t < 6; ++t) sc->hforms[t] = s[t];
}

struct EnergyParams {
    double alpha, alphaH, U, StepAlternative;
    int64_t numS;
    // mixed precision only: a step below 1 whose predicted gain over step 1, c2 (1 - s)^2, is below
    // oda_noise |E_tot| is noise of the FP32-level P_new, and step 1 is taken (0: the reference rule)
    double oda_noise;
    double fixed_step;   // mode 2 (linear mixing): the step, in place of OptimalStep's
};

// energies of the state (1-s) a + s b from the forms
__device__ inline void energies_at(const ScfScalars* sc, double s, double E[4]) {
    const double u = 1.0 - s;
    E[0] = u * sc->forms[0] + s * sc->forms[1];
    E[1] = -0.5 * (u * u * sc->forms[2] + 2.0 * u * s * sc->forms[3] + s * s * sc->forms[4]);
    // GetHartreeHubbardEnergy with dens1 = dens2 = dn: fsumH = 2 dn.LR.dn, fsumU = dn.dn
    E[2] = 2.0 * (u * u * sc->hforms[0] + 2.0 * u * s * sc->hforms[1] + s * s * sc->hforms[2]);
    E[3] = u * u * sc->hforms[3] + 2.0 * u * s * sc->hforms[4] + s * s * sc->hforms[5];
}
__device__ inline double total_energy(const EnergyParams& p, const double E[4]) {
    // Main.f90:312 / 556
    return p.alpha * E[1] * (double)(3 - p.numS) + E[0] * (double)(3 - p.numS) + p.U * E[3] + p.alphaH * E[2];
}

// mode 0: OptimalStep; mode 1: energies of b only (s = 1); mode 2: linear mixing with p.fixed_step
__global__ void k_oda(ScfScalars* sc, EnergyParams p, int mode) {
    if (threadIdx.x != 0) return;
    double E1[4], Eh[4], Es[4];
    energies_at(sc, 1.0, E1);
    if (mode == 1) {
        for (int t = 0; t < 4; ++t) sc->Eout[t] = E1[t];
        sc->Etot_in = total_energy(p, sc->Ein);
        sc->Etot_out = total_energy(p, E1);
        sc->step = 1.0;
        return;
    }
    const double c0 = total_energy(p, sc->Ein);
    const double t1 = total_energy(p, E1);
    energies_at(sc, 0.5, Eh);
    const double t2 = total_energy(p, Eh);
    const double c1 = 4.0 * t2 - t1 - 3.0 * c0;
    const double c2 = t1 - c0 - c1;
    double step;
    if (mode == 2)
        step = p.fixed_step;
    else if ((c2 > 0) && (fabs(-c1 / 2.0 / c2 - .5) < 0.5))
        step = -c1 / 2.0 / c2;
    else if (t1 < c0)
        step = 1.0;
    else
        step = p.StepAlternative;
    if (mode == 0 && p.oda_noise > 0.0 && step < 1.0 && c2 * (1.0 - step) * (1.0 - step) < p.oda_noise * fabs(c0))
        step = 1.0;
    energies_at(sc, step, Es);
    for (int t = 0; t < 4; ++t) sc->Eout[t] = Es[t];
    sc->E1tot = t1;
    sc->Ehtot = t2;
    sc->Etot_in = c0;
    sc->Etot_out = total_energy(p, Es);
    sc->step = step;
}

// Diagonal part of the mix, run before k_mix_p: density of the mixed state, |n - n_in|,
// potential V = 2 alphaH LR dn + U dn from the two matvecs (Main.f90:560-585).
__global__ void __launch_bounds__(256) k_mix_dens(const double2* __restrict__ P, const double2* __restrict__ Pn,
                                                  int64_t N, const ScfScalars* __restrict__ sc,
                                                  double* __restrict__ dens, double* __restrict__ V,
                                                  const double* __restrict__ y, double alphaH, double U,
                                                  double* __restrict__ mpart) {
    const double s = sc->step, u = 1.0 - s;
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double dn = 0.0, dv = 0.0;
    if (n < N) {
        const double2 a = P[n + (size_t)n * N], b = Pn[n + (size_t)n * N];
        const double d_new = s * b.x + u * a.x;
        dn = fabs(d_new - dens[n]);
        dens[n] = d_new;
        const double v = 2.0 * alphaH * (u * y[n] + s * y[N + n]) + U * (d_new - 0.5);
        dv = fabs(v - V[n]);
        V[n] = v;
    }
    __shared__ double sh[32];
    double r0 = block_max(dn, sh), r1 = block_max(dv, sh);
    if (threadIdx.x == 0) {
        mpart[blockIdx.x * 2] = r0;
        mpart[blockIdx.x * 2 + 1] = r1;
    }
}

__global__ void k_mix_finish(const double* __restrict__ mpart, int nparts, ScfScalars* sc) {
    if (threadIdx.x != 0) return;
    double dn = 0.0, dv = 0.0;
    for (int q = 0; q < nparts; ++q) {
        dn = fmax(dn, mpart[2 * q]);
        dv = fmax(dv, mpart[2 * q + 1]);
    }
    sc->dn_max = dn;
    sc->dV_max = dv;
    sc->residual = fmax(dv, sc->step * sc->forms[5]);
    for (int t = 0; t < 4; ++t) sc->Ein[t] = sc->Eout[t];
}

// P <- s Pnew + (1-s) P  (zFock = Step*zFock + (1-Step)*zFockIn, Main.f90:558; zFockIn = zFock)
__global__ void __launch_bounds__(256) k_mix_p(double2* __restrict__ P, const double2* __restrict__ Pn, size_t total,
                                               const ScfScalars* __restrict__ sc) {
    const double s = sc->step, u = 1.0 - s;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
        const double2 a = P[q], b = Pn[q];
        P[q] = make_double2(s * b.x + u * a.x, s * b.y + u * a.y);
    }
}

// P_new = (win + bulk) / Nk   (Main.f90:510-511)
__global__ void __launch_bounds__(256) k_combine(double2* __restrict__ win, const double2* __restrict__ bulk,
                                                 size_t total, double Nk) {
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total; q += (size_t)gridDim.x * blockDim.x) {
        const double2 a = win[q], b = bulk[q];
        win[q] = make_double2((a.x + b.x) / Nk, (a.y + b.y) / Nk);
    }
}

// density Re diag P(:,:,1)
__global__ void k_density(const double2* __restrict__ P, int64_t N, double* __restrict__ dens) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n < N) dens[n] = P[n + (size_t)n * N].x;
}

// V = 2 alphaH y + U dn (single-state potential, Main.f90:319-327)
__global__ void k_potential(const double* __restrict__ y, const double* __restrict__ dens, int64_t N, double alphaH,
                            double U, double* __restrict__ V) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (n < N) V[n] = 2.0 * alphaH * y[n] + U * (dens[n] - 0.5);
}

// ---------------------------------------------------------------- host launchers
int scf_energy_forms(Context& c, const double* te, const double2* Pa, const double2* Pb, const double* da,
                     const double* db, double* y, double* work, ScfScalars* sc) {
    const int64_t N = c.N;
    const double NN = (double)N * N;
    prof_begin(ST_ENERGY);
    k_energy_pass<<<RED_CTAS, 256, 0, c.stream>>>(te, Pa, Pb, N, c.s.alpha, work);
    FORGE_LAUNCH_CHECK();
    k_reduce_forms<<<1, 32, 0, c.stream>>>(work, RED_CTAS, sc);
    FORGE_LAUNCH_CHECK();
    // 8 tables + two 4-cell complex states read once
    prof_end(ST_ENERGY, 8.0 * NN * 8.0 + 2.0 * 4.0 * NN * 16.0, 4.0 * NN * 14.0);
    double* part = work + RED_CTAS * 8;
    dim3 g((unsigned)((N + 255) / 256), LR_CHUNKS);
    prof_begin(ST_LRMATVEC);
    k_lr_matvec<<<g, 256, 0, c.stream>>>(c.LR.as<double>(), da, db, N, part);
    FORGE_LAUNCH_CHECK();
    prof_end(ST_LRMATVEC, NN * 8.0, 4.0 * NN);
    double* hpart = part + (size_t)LR_CHUNKS * 2 * N;
    const unsigned nb = (unsigned)((N + 255) / 256);
    k_lr_finish<<<nb, 256, 0, c.stream>>>(part, da, db, N, y, hpart);
    FORGE_LAUNCH_CHECK();
    k_reduce_hforms<<<1, 32, 0, c.stream>>>(hpart, (int)nb, sc);
    FORGE_LAUNCH_CHECK();
    return 0;
}

size_t scf_work_doubles(int64_t N) { return RED_CTAS * 8 + (size_t)LR_CHUNKS * 2 * N + 8 * ((N + 255) / 256) + 64; }

int scf_oda(Context& c, ScfScalars* sc, int mode, double fixed_step) {
    // the FP32-noise guard of OptimalStep only for FP32-accurate P_new (not after the refinement)
    EnergyParams p{c.s.alpha, c.s.alphaH, c.s.U, c.s.StepAlternative, 1,
                   (c.precision == FORGE_PREC_MIXED && !c.refined) ? 1e-8 : 0.0, fixed_step};
    k_oda<<<1, 32, 0, c.stream>>>(sc, p, mode);
    FORGE_LAUNCH_CHECK();
    return 0;
}

int scf_mix(Context& c, double2* P, const double2* Pn, double* dens, double* V, const double* y, double* work,
            ScfScalars* sc) {
    const int64_t N = c.N;
    const unsigned nb = (unsigned)((N + 255) / 256);
    k_mix_dens<<<nb, 256, 0, c.stream>>>(P, Pn, N, sc, dens, V, y, c.s.alphaH, c.s.U, work);
    FORGE_LAUNCH_CHECK();
    k_mix_finish<<<1, 32, 0, c.stream>>>(work, (int)nb, sc);
    FORGE_LAUNCH_CHECK();
    prof_begin(ST_MIX);
    k_mix_p<<<1216, 256, 0, c.stream>>>(P, Pn, 4 * (size_t)N * N, sc);
    FORGE_LAUNCH_CHECK();
    prof_end(ST_MIX, 3.0 * 4.0 * (double)N * N * 16.0, 0.0);
    return 0;
}

int scf_combine(Context& c, double2* win, const double2* bulk) {
    k_combine<<<1216, 256, 0, c.stream>>>(win, bulk, 4 * (size_t)c.N * c.N, (double)c.Nk);
    FORGE_LAUNCH_CHECK();
    return 0;
}

// ---------------------------------------------------------------- Pulay / Anderson mixing
// State x = P_in (4 cells, FP64), residual r = P_new - P_in.  The history holds, per slot,
// dX_i = x_{i+1} - x_i and dR_i = r_{i+1} - r_i in complex64: both are small near convergence, so
// their FP32 rounding is relative to their own size; x and r themselves stay FP64.
constexpr int DIIS_CTAS = 1216;

// dR_new = (Pn - P) - rprev into slot snew; a_i = Re<dR_i, dR_new>, b_i = Re<dR_i, r> for the
// slots in the list (snew included, with the value just stored); per-CTA partials [2 x DIIS_MAX].
__global__ void __launch_bounds__(256) k_diis_dots(DiisArgs d) {
    double a[DIIS_MAX], bb[DIIS_MAX];
#pragma unroll
    for (int i = 0; i < DIIS_MAX; ++i) a[i] = bb[i] = 0.0;
    float2* dRnew = d.hist + (size_t)(2 * d.snew + 1) * d.nn4;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < d.nn4; q += (size_t)gridDim.x * blockDim.x) {
        const double2 x = d.P[q], y = d.Pn[q];
        const double rr = y.x - x.x, ri = y.y - x.y;
        const float2 rp = d.rprev[q];
        const float2 dn = make_float2((float)(rr - (double)rp.x), (float)(ri - (double)rp.y));
        dRnew[q] = dn;
#pragma unroll
        for (int i = 0; i < DIIS_MAX; ++i) {
            if (i < d.nslots) {
                const float2 v = (d.slots[i] == d.snew) ? dn : d.hist[(size_t)(2 * d.slots[i] + 1) * d.nn4 + q];
                a[i] += (double)v.x * dn.x + (double)v.y * dn.y;
                bb[i] += (double)v.x * rr + (double)v.y * ri;
            }
        }
    }
    __shared__ double sh[32];
#pragma unroll
    for (int i = 0; i < DIIS_MAX; ++i) {
        if (i < d.nslots) {   // uniform over the block
            const double sa = block_sum(a[i], sh);
            if (threadIdx.x == 0) d.part[(size_t)blockIdx.x * 2 * DIIS_MAX + i] = sa;
            const double sb = block_sum(bb[i], sh);
            if (threadIdx.x == 0) d.part[(size_t)blockIdx.x * 2 * DIIS_MAX + DIIS_MAX + i] = sb;
        }
    }
}

// x_next = P + beta r - sum_i g_i (dX_i + beta dR_i); dX into slot spend; rprev = r; P = x_next
__global__ void __launch_bounds__(256) k_diis_update(DiisArgs d) {
    float2* dXp = d.hist + (size_t)(2 * d.spend) * d.nn4;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < d.nn4; q += (size_t)gridDim.x * blockDim.x) {
        const double2 x = d.P[q], y = d.Pn[q];
        const double rr = y.x - x.x, ri = y.y - x.y;
        double nx = x.x + d.beta * rr, ny = x.y + d.beta * ri;
#pragma unroll
        for (int i = 0; i < DIIS_MAX; ++i) {
            if (i < d.nslots) {
                const float2 dx = d.hist[(size_t)(2 * d.slots[i]) * d.nn4 + q];
                const float2 dr = d.hist[(size_t)(2 * d.slots[i] + 1) * d.nn4 + q];
                nx -= d.gamma[i] * ((double)dx.x + d.beta * (double)dr.x);
                ny -= d.gamma[i] * ((double)dx.y + d.beta * (double)dr.y);
            }
        }
        dXp[q] = make_float2((float)(nx - x.x), (float)(ny - x.y));
        d.rprev[q] = make_float2((float)rr, (float)ri);
        d.P[q] = make_double2(nx, ny);
    }
}

// residual of the state before mixing: max(|V(P_new) - V(P_in)|, max alpha |fv| |P_new - P_in|),
// from the LR products y = [LR (d_in - 1/2), LR (d_new - 1/2)] of the (P_in, P_new) energy pass
__global__ void __launch_bounds__(256) k_diis_residual(const double* __restrict__ y, const double* __restrict__ din,
                                                       const double* __restrict__ dnew, int64_t N, double alphaH,
                                                       double U, double* __restrict__ mpart) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double dv = 0.0;
    if (n < N) dv = fabs(2.0 * alphaH * (y[N + n] - y[n]) + U * (dnew[n] - din[n]));
    __shared__ double sh[32];
    const double r = block_max(dv, sh);
    if (threadIdx.x == 0) mpart[blockIdx.x] = r;
}

// density of the mixed state and max |n - n_in|
__global__ void __launch_bounds__(256) k_diis_dens(const double2* __restrict__ P, int64_t N, double* __restrict__ dens,
                                                   double* __restrict__ mpart) {
    const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double dn = 0.0;
    if (n < N) {
        const double d = P[n + (size_t)n * N].x;
        dn = fabs(d - dens[n]);
        dens[n] = d;
    }
    __shared__ double sh[32];
    const double r = block_max(dn, sh);
    if (threadIdx.x == 0) mpart[blockIdx.x] = r;
}

__global__ void k_diis_finish(const double* __restrict__ rpart, const double* __restrict__ dpart, int nparts,
                              ScfScalars* sc, int stage) {
    if (threadIdx.x != 0) return;
    double m = 0.0;
    for (int q = 0; q < nparts; ++q) m = fmax(m, stage == 0 ? rpart[q] : dpart[q]);
    if (stage == 0) {
        sc->dV_max = m;
        sc->residual = fmax(m, sc->forms[5]);
    } else if (stage == 1) {
        sc->dn_max = m;
    } else {
        for (int t = 0; t < 4; ++t) sc->Ein[t] = sc->Eout[t];
    }
}

int scf_diis_dots(Context& c, const DiisArgs& d) {
    k_diis_dots<<<DIIS_CTAS, 256, 0, c.stream>>>(d);
    FORGE_LAUNCH_CHECK();
    return 0;
}

int scf_diis_update(Context& c, const DiisArgs& d) {
    prof_begin(ST_MIX);
    k_diis_update<<<DIIS_CTAS, 256, 0, c.stream>>>(d);
    FORGE_LAUNCH_CHECK();
    prof_end(ST_MIX, (double)d.nn4 * (16.0 * 3.0 + 8.0 * 2.0 + 16.0 * d.nslots), 0.0);
    return 0;
}

int scf_diis_residual(Context& c, const double* y, const double* din, const double* dnew, double* work,
                      ScfScalars* sc) {
    const unsigned nb = (unsigned)((c.N + 255) / 256);
    k_diis_residual<<<nb, 256, 0, c.stream>>>(y, din, dnew, c.N, c.s.alphaH, c.s.U, work);
    FORGE_LAUNCH_CHECK();
    k_diis_finish<<<1, 32, 0, c.stream>>>(work, work, (int)nb, sc, 0);
    FORGE_LAUNCH_CHECK();
    return 0;
}

int scf_diis_dens(Context& c, const double2* P, double* dens, double* work, ScfScalars* sc) {
    const unsigned nb = (unsigned)((c.N + 255) / 256);
    k_diis_dens<<<nb, 256, 0, c.stream>>>(P, c.N, dens, work);
    FORGE_LAUNCH_CHECK();
    k_diis_finish<<<1, 32, 0, c.stream>>>(work, work, (int)nb, sc, 1);
    FORGE_LAUNCH_CHECK();
    return 0;
}

int scf_diis_commit(Context& c, ScfScalars* sc) {
    k_diis_finish<<<1, 32, 0, c.stream>>>(nullptr, nullptr, 0, sc, 2);
    FORGE_LAUNCH_CHECK();
    return 0;
}

size_t scf_diis_parts() { return (size_t)DIIS_CTAS * 2 * DIIS_MAX; }

int scf_density(Context& c, const double2* P, double* dens) {
    k_density<<<(unsigned)((c.N + 255) / 256), 256, 0, c.stream>>>(P, c.N, dens);
    FORGE_LAUNCH_CHECK();
    return 0;
}

int scf_potential(Context& c, const double* y, const double* dens, double* V) {
    k_potential<<<(unsigned)((c.N + 255) / 256), 256, 0, c.stream>>>(y, dens, c.N, c.s.alphaH, c.s.U, V);
    FORGE_LAUNCH_CHECK();
    return 0;
}

}  // namespace forge
