// C-ABI entry points (include/forge_gpu.h): one per reference routine of the SCF
// path, plus a fused device-resident iteration.  Host code here is compiled with
// -ffp-contract=off so that the k.R phases follow the reference's unfused dot product.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "eig.cuh"
#include "proj.cuh"

namespace forge {

static thread_local std::string g_err;
static thread_local int g_errcode = 0;

void set_error(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    g_errcode = code;
}
int last_error_code() { return g_errcode; }

static std::atomic<int64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int DevBuf::ensure(size_t nbytes) {
    if (nbytes <= bytes && ptr) return 0;
    release();
    if (nbytes == 0) return 0;
    cudaError_t e = cudaMalloc(&ptr, nbytes);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        set_error(FORGE_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", nbytes, cudaGetErrorString(e));
        return FORGE_ERR_NOMEM;
    }
    bytes = nbytes;
    return 0;
}
void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

// defined in scf.cu
int build_energy_tables(Context& c, DevBuf& te);
int launch_sort_fermi(Context& c, const double* w, double nfilling, double* sorted_e, int64_t* sorted_idx,
                      WinState* states, ScfScalars* sc);
int scf_energy_forms(Context& c, const double* te, const double2* Pa, const double2* Pb, const double* da,
                     const double* db, double* y, double* work, ScfScalars* sc);
size_t scf_work_doubles(int64_t N);
int scf_oda(Context& c, ScfScalars* sc, int mode, double fixed_step = 0.0);
int scf_mix(Context& c, double2* P, const double2* Pn, double* dens, double* V, const double* y, double* work,
            ScfScalars* sc);
int scf_combine(Context& c, double2* win, const double2* bulk);
int scf_density(Context& c, const double2* P, double* dens);
int scf_potential(Context& c, const double* y, const double* dens, double* V);
int scf_diis_dots(Context& c, const DiisArgs& d);
int scf_diis_update(Context& c, const DiisArgs& d);
int scf_diis_residual(Context& c, const double* y, const double* din, const double* dnew, double* work,
                      ScfScalars* sc);
int scf_diis_dens(Context& c, const double2* P, double* dens, double* work, ScfScalars* sc);
int scf_diis_commit(Context& c, ScfScalars* sc);
size_t scf_diis_parts();
// mixed-precision eigen-solver (eig_mixed.cu) and its FP64 window refinement (rr_window.cu)
int eig_mixed(cudaStream_t st, EigArgs& g, void* mixed_ws);
size_t eig_mixed_workspace_bytes(int64_t n, int64_t iu, int64_t batch);
int rr_window(cudaStream_t st, const double2* H, int64_t strideH, double2* X, int64_t ldx, int64_t strideX, double* w,
              int64_t iu, int64_t n, int64_t c0, int64_t nw, int64_t batch, void* ws);
size_t rr_window_workspace_bytes(int64_t n, int64_t batch);
const float* eig_mixed_planes(void* mixed_ws, int64_t n, int64_t iu, int64_t batch, int64_t* n4);
size_t oa_workspace_bytes(int64_t n, int64_t iu);
int launch_pad_slot(cudaStream_t st, const double2* src, int64_t nb, double2* dst, int64_t n, double* rowsum,
                    double* sigma);
int oa_refine(cudaStream_t st, double2* H, int64_t strideH, const float* Xs, int64_t n4, int64_t nall,
              const double* lam, int64_t n, int64_t iu, int64_t batch, double2* X, int64_t ldx, int64_t strideX,
              double* w_out, int64_t w_stride, void* ws, int* err, double delta, int depth);

}  // namespace forge

using namespace forge;

struct forge_ctx {
    Context c;
    Profiler prof;
    cudaEvent_t marks[64] = {};
    DevBuf te;           // energy tables
    DevBuf Pn, win;      // P_new, window accumulator / scratch
    DevBuf eigws, mixws; // eigen-solver workspaces
    DevBuf states, sorted_e, sorted_idx, sc, work, y, dens_new, w;
    DevBuf projws, tcerr;  // tensor-core projector staging and its error flag
    DevBuf rrws;           // FP64 window refinement of the mixed path
    DevBuf pstates;        // partially occupied states of the fused projector
    int64_t rr_width = 32; // bands refined in FP64 after each mixed solve (0: off)
    // eigenpair refinement of the mixed solve (forge_gpu_set_eigen_refinement): mode 0 off, 1 every
    // mixed solve, 2 once the last SCF residual is below oa_below
    int oa_mode = 0;
    double oa_below = 0.0, oa_delta = 1e-3;
    int oa_depth = 4;
    bool oa_active = false, oa_latched = false;
    double last_residual = INFINITY;
    DevBuf oaws, w_all;
    // group solve led by this context (forge_gpu_solve_group): padded H slots, eigenpairs, workspaces
    DevBuf g_H, g_X, g_w, g_eigws, g_mixws, g_tmp, g_rows, g_sig, g_rr;
    int64_t eig_batch = 0;
    int64_t k_begin = 0, k_end = 0;  // local k range (k_end = 0: all k)
    // mixing: FORGE_MIX_ODA (OptimalStep, the reference), FORGE_MIX_PULAY (Anderson / Pulay) or
    // FORGE_MIX_LINEAR (P = beta P_new + (1 - beta) P_in)
    int mix_mode = FORGE_MIX_ODA;
    int diis_depth = 6;
    double diis_beta = 0.7;
    DevBuf diis_hist, diis_rprev, diis_part;
    std::vector<int> diis_order;     // complete history slots, oldest first
    int diis_pending = -1;           // slot holding dX of the last step (its dR comes next iteration)
    int diis_nslots = 0;             // slots allocated (depth + 1)
    bool diis_has_prev = false;
    double diis_G[DIIS_MAX][DIIS_MAX] = {};
    // C3-reduced solve (forge_gpu_set_c3): H(k) solved for the first k of each C3 orbit only
    bool c3 = false;
    C3Tables c3t;
    DevBuf c3_Xr, c3_wr, c3_tab, c3_perm, c3_phase;
    // symmetry switches applied to P_new in the fused iteration (forge_gpu_set_symmetry)
    bool sym_T = false, sym_C2 = false, sym_C2T = false;
    DevBuf c2_perm;
    // valley projection (forge_gpu_set_valley): V(k) terms, per-k phases, and the transform buffers
    bool valley = false;
    DevBuf v_rowp, v_col, v_coef, v_code, v_ph, v_W, v_G, v_S, v_Xv, v_st;
    bool have_solve = false, have_sort = false, have_pnew = false, have_state = false, bulk_is_fused = false;
    std::vector<int64_t> h_sorted_idx;
    std::vector<double2> h_bph;
};

namespace {

int read_scalars(forge_ctx* x, ScfScalars* h);
void diis_reset(forge_ctx* x);

int check_ctx(forge_ctx* x) {
    if (!x) {
        set_error(FORGE_ERR_ARG, "null context");
        return FORGE_ERR_ARG;
    }
    x->prof.stream = x->c.stream;
    set_current_profiler(&x->prof);
    return 0;
}

int choose_batch(forge_ctx* x) {
    Context& c = x->c;
    const int64_t N = c.N, iu = c.nUpper;
    const bool oa = c.precision == FORGE_PREC_MIXED && x->oa_mode != 0;
    const int64_t iu_solve = oa ? N : iu;   // the refinement needs every eigenpair of the mixed solve
    size_t per_k = (size_t)N * N * 16 + eig_workspace_bytes(N, iu_solve, 1);
    if (c.precision == FORGE_PREC_MIXED) per_k += eig_mixed_workspace_bytes(N, iu_solve, 1);
    if (oa) per_k += (size_t)N * 8;
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    // kept free: 8 GB headroom, the eigenvectors of every k, the four bulk cells and the
    // projector / window work arrays allocated after the batch is chosen
    const int64_t xslots = x->c3 ? x->c3t.nslots + (int64_t)x->c3t.reps.size() : c.Nk;
    // the Pulay history (depth + 1 slots of dX, dR and the previous residual, complex64 over the four
    // cells) is allocated at the first mixing step, after this choice
    const size_t diis = x->mix_mode == FORGE_MIX_PULAY ? ((size_t)(2 * (x->diis_depth + 1) + 1) * 4 * N * N * 8) : 0;
    const size_t reserve = ((size_t)8 << 30) + (size_t)xslots * N * iu * 16 + (size_t)10 * N * N * 16 +
                           (oa ? oa_workspace_bytes(N, iu) : 0) + diis;
    const size_t budget = freeb > reserve ? freeb - reserve : freeb / 4;
    int64_t b = (int64_t)(budget / per_k);
    // FORGE_EIG_BATCH caps the number of k points solved per launch (memory control)
    if (const char* env = std::getenv("FORGE_EIG_BATCH")) {
        const long cap = std::strtol(env, nullptr, 10);
        if (cap > 0 && cap < b) b = cap;
    }
    if (b < 1) b = 1;
    if (b > c.Nk) b = c.Nk;
    // equal batches: ceil(Nk / b) launches of (nearly) the same size
    const int64_t nbatches = (c.Nk + b - 1) / b;
    b = (c.Nk + nbatches - 1) / nbatches;
    return (int)b;
}

int ensure_solve_buffers(forge_ctx* x) {
    Context& c = x->c;
    const int64_t N = c.N, iu = c.nUpper, Nk = c.Nk;
    const size_t NN = (size_t)N * N;
    if (x->eig_batch == 0) x->eig_batch = choose_batch(x);
    const int64_t B = x->eig_batch;
    // eigenvector slots: one per k, plus the two rotated copies of each C3-invariant k
    const int64_t nslots = x->c3 ? x->c3t.nslots : Nk;
    FORGE_TRY(c.H.ensure((size_t)B * NN * sizeof(double2)));
    FORGE_TRY(c.X.ensure((size_t)nslots * N * iu * sizeof(double2)));
    FORGE_TRY(x->w.ensure((size_t)nslots * iu * sizeof(double)));
    if (x->c3) {
        const size_t nr = x->c3t.reps.size();
        FORGE_TRY(x->c3_Xr.ensure(nr * N * iu * sizeof(double2)));
        FORGE_TRY(x->c3_wr.ensure(nr * iu * sizeof(double)));
    }
    const bool oa = c.precision == FORGE_PREC_MIXED && x->oa_mode != 0;
    const int64_t iu_solve = oa ? N : iu;
    FORGE_TRY(x->eigws.ensure(eig_workspace_bytes(N, iu_solve, B)));
    if (c.precision == FORGE_PREC_MIXED) FORGE_TRY(x->mixws.ensure(eig_mixed_workspace_bytes(N, iu_solve, B)));
    if (oa) {
        FORGE_TRY(x->w_all.ensure((size_t)B * N * sizeof(double)));
        FORGE_TRY(x->oaws.ensure(oa_workspace_bytes(N, iu)));
        FORGE_TRY(x->tcerr.ensure(sizeof(int)));
    }
    FORGE_TRY(c.bulk.ensure(4 * NN * sizeof(double2)));
    return 0;
}

int upload_state(forge_ctx* x, const double* Potential, const double* zFock) {
    Context& c = x->c;
    const size_t NN = (size_t)c.N * c.N;
    if (Potential) FORGE_CUDA(cudaMemcpyAsync(c.V.ptr, Potential, c.N * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    if (zFock) {
        FORGE_CUDA(cudaMemcpyAsync(c.P.ptr, zFock, 4 * NN * sizeof(double2), cudaMemcpyHostToDevice, c.stream));
        x->have_state = true;
    }
    return 0;
}

// eigen-solve of the batch of H already assembled in c.H for k in [k0, k0+nb); the eigenpairs go to
// the slots of those k, or to Xdst / wdst when given
int eig_batch_run(forge_ctx* x, int64_t k0, int64_t nb, int* info, double2* Xdst = nullptr, double* wdst = nullptr) {
    Context& c = x->c;
    const int64_t N = c.N, iu = c.nUpper;
    EigArgs g{};
    g.n = N;
    g.iu = iu;
    g.batch = nb;
    g.A = c.H.as<double2>();
    g.lda = N;
    g.strideA = N * N;
    g.X = Xdst ? Xdst : c.X.as<double2>() + (size_t)k0 * N * iu;
    g.ldx = N;
    g.strideX = N * iu;
    g.w = wdst ? wdst : x->w.as<double>() + (size_t)k0 * iu;
    g.ortol_rel = 1e-7;
    const bool oa = c.precision == FORGE_PREC_MIXED && x->oa_active;
    double* w_iu = g.w;
    if (oa) {
        // every eigenpair of the mixed solve; FP64 columns 1..iu, eigenvalues of all N in w_all
        g.iu = N;
        g.iu_out = iu;
        g.w = x->w_all.as<double>();
    }
    eig_bind_workspace(g, x->eigws.ptr);
    if (c.precision == FORGE_PREC_MIXED) {
        auto solve = [&]() -> int {
            int r = eig_mixed(c.stream, g, x->mixws.ptr);
            if (r || !oa) return r;
            // FP64-accurate eigenpairs 1..iu from the mixed ones (tensor-core refinement)
            int64_t n4 = 0;
            const float* planes = eig_mixed_planes(x->mixws.ptr, N, N, nb, &n4);
            FORGE_CUDA(cudaMemsetAsync(x->tcerr.ptr, 0, sizeof(int), c.stream));
            r = oa_refine(c.stream, g.A, g.strideA, planes, n4, N, g.w, N, iu, nb, g.X, g.ldx, g.strideX, w_iu, iu,
                          x->oaws.ptr, x->tcerr.as<int>(), x->oa_delta, x->oa_depth);
            if (r) return r;
            int herr = 0;
            FORGE_CUDA(cudaMemcpyAsync(&herr, x->tcerr.ptr, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            FORGE_CUDA(cudaStreamSynchronize(c.stream));
            if (herr) {
                set_error(FORGE_ERR_TIMEOUT, "tcgen05 GEMM of the eigenpair refinement: a bounded mbarrier wait gave up");
                return FORGE_ERR_TIMEOUT;
            }
            return 0;
        };
        int rc = solve();
        if (rc == FORGE_ERR_TIMEOUT) {
            // a bounded tensor-core wait gave up (the kernel drained and freed its TMEM): the
            // input H(k) is unchanged (the refinement only mirrors its lower triangle), so the
            // batch is solved again once
            std::fprintf(stderr, "forge: %s; solving the batch again\n", forge_gpu_last_error());
            rc = solve();
        }
        FORGE_TRY(rc);
        g.w = w_iu;
        g.iu = iu;
        if (x->rr_width > 0) {
            // FP64 Rayleigh-Ritz on the top rr_width computed bands (the window around the Fermi level)
            const int64_t nw = std::min<int64_t>(x->rr_width, iu);
            FORGE_TRY(x->rrws.ensure(rr_window_workspace_bytes(N, nb)));
            FORGE_TRY(rr_window(c.stream, g.A, g.strideA, g.X, g.ldx, g.strideX, g.w, iu, N, iu - nw, nw, nb,
                                x->rrws.ptr));
        }
    } else {
        FORGE_TRY(eig_fp64(c.stream, g));
    }
    std::vector<int> fails(nb);
    FORGE_CUDA(cudaMemcpyAsync(fails.data(), g.fail, nb * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    int bad = 0;
    for (int64_t b = 0; b < nb; ++b) bad += fails[b] ? 1 : 0;
    *info += bad;
    return 0;
}

// bulk_c += ph_c(k) conj(X_k) X_k^T over the first K columns (precision of the context)
int project_k(forge_ctx* x, int64_t k, int64_t K, const double2* ph, double2* out) {
    Context& c = x->c;
    const int64_t N = c.N, iu = c.nUpper;
    const double2* Xk = c.X.as<double2>() + (size_t)k * N * iu;
    if (c.precision == FORGE_PREC_MIXED) {
        FORGE_TRY(x->tcerr.ensure(sizeof(int)));
        if (x->oa_active) {
            // refined eigenvectors: the projector keeps their FP64 accuracy (exact sliced products)
            FORGE_TRY(x->projws.ensure(proj_tc_exact_workspace_bytes(N, iu)));
            return bulk_projector_tc_exact(c.stream, Xk, N, N, K, iu, ph, out, x->projws.ptr, x->tcerr.as<int>());
        }
        FORGE_TRY(x->projws.ensure(proj_tc_workspace_floats(N, iu) * sizeof(float)));
        return bulk_projector_tc(c.stream, Xk, N, N, K, iu, ph, out, x->projws.as<float>(), x->tcerr.as<int>());
    }
    return bulk_projector_fp64(c.stream, Xk, N, N, K, ph, out);
}

// project_k, with the average of Solve_C3 / GetFock_C3 at a C3-invariant k: the projector of k's
// eigenvectors and of their two rotated copies, each with a third of the phases
int project_k_c3(forge_ctx* x, int64_t k, int64_t K, const double2* ph, double2* out) {
    if (!x->c3 || x->c3t.extra[k] < 0) return project_k(x, k, K, ph, out);
    double2 ph3[4];
    for (int t = 0; t < 4; ++t) ph3[t] = cscale(ph[t], 1.0 / 3.0);
    const int64_t e = x->c3t.extra[k];
    FORGE_TRY(project_k(x, k, K, ph3, out));
    FORGE_TRY(project_k(x, e, K, ph3, out));
    return project_k(x, e + 1, K, ph3, out);
}

// window states with the C3 average: a state at a C3-invariant k becomes itself and its two
// rotated copies, each with a third of its weighted phases (GetFock_C3, HartreeFock.f90:650-876)
void expand_c3_states(forge_ctx* x, std::vector<WinState>& st) {
    if (!x->c3) return;
    std::vector<WinState> out;
    out.reserve(st.size());
    for (const WinState& s0 : st) {
        const int64_t e = x->c3t.extra[s0.k];
        if (e < 0) {
            out.push_back(s0);
            continue;
        }
        WinState s = s0;
        for (int t = 0; t < 4; ++t) s.wph[t] = cscale(s0.wph[t], 1.0 / 3.0);
        out.push_back(s);
        s.k = e;
        out.push_back(s);
        s.k = e + 1;
        out.push_back(s);
    }
    st.swap(out);
}

// full Solve on the device: H(k), eigenpairs, and (with_projector) the bulk projector of bands
// 1..nLower-1 (not divided by Nk), as Solve returns it
int solve_device(forge_ctx* x, int* info, bool with_projector = true) {
    Context& c = x->c;
    // mode 2 latches: once an SCF residual fell below oa_below, every later solve of that SCF
    // (until the next guess or state load) is refined
    if (x->oa_mode == 2 && x->last_residual < x->oa_below) x->oa_latched = true;
    const bool was_active = x->oa_active;
    x->oa_active = c.precision == FORGE_PREC_MIXED && (x->oa_mode == 1 || (x->oa_mode == 2 && x->oa_latched));
    c.refined = x->oa_active;
    // the Pulay history of FP32-accurate iterations holds their noise: the refined iterations start
    // a new one (as a change of precision does)
    if (x->oa_active && !was_active) diis_reset(x);
    FORGE_TRY(ensure_solve_buffers(x));
    const int64_t N = c.N, Nk = c.Nk, B = x->eig_batch;
    const size_t NN = (size_t)N * N;
    FORGE_CUDA(cudaMemsetAsync(c.bulk.ptr, 0, 4 * NN * sizeof(double2), c.stream));
    *info = 0;
    x->h_bph.resize(Nk * 4);
    FORGE_CUDA(cudaMemcpyAsync(x->h_bph.data(), c.bphase.ptr, Nk * 4 * sizeof(double2), cudaMemcpyDeviceToHost,
                               c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    if (x->tcerr.ptr) FORGE_CUDA(cudaMemsetAsync(x->tcerr.ptr, 0, sizeof(int), c.stream));
    // local k range of this rank (all k unless forge_gpu_set_kshard narrowed it)
    const int64_t kb = x->k_begin, ke = (x->k_end > 0) ? x->k_end : Nk;
    if (x->c3) {
        if (kb != 0 || ke != Nk) {
            set_error(FORGE_ERR_STATE, "the C3-reduced solve runs over the whole k grid (no k shard)");
            return FORGE_ERR_STATE;
        }
        // Solve_C3 (HartreeFock.f90:189-216): the orbit representatives in batches, then the rotated
        // eigenvectors and the copied bands of every k
        const int64_t N_ = c.N, iu = c.nUpper, nr = (int64_t)x->c3t.reps.size();
        for (int64_t r0 = 0; r0 < nr; r0 += B) {
            const int64_t nb = (nr - r0 < B) ? nr - r0 : B;
            for (int64_t b = 0; b < nb; ++b)
                FORGE_TRY(launch_assemble(c, c.V.as<double>(), c.P.as<double2>(), x->c3t.reps[r0 + b], 1,
                                          c.H.as<double2>() + (size_t)b * NN));
            FORGE_TRY(eig_batch_run(x, r0, nb, info, x->c3_Xr.as<double2>() + (size_t)r0 * N_ * iu,
                                    x->c3_wr.as<double>() + (size_t)r0 * iu));
        }
        FORGE_TRY(launch_c3_rotate(c.stream, x->c3_Xr.as<double2>(), x->c3_wr.as<double>(), N_, iu, x->c3t.nslots,
                                   x->c3_tab.as<int64_t>(), x->c3_perm.as<int64_t>(), x->c3_phase.as<double2>(),
                                   c.X.as<double2>(), x->w.as<double>()));
        if (with_projector)
            for (int64_t k = 0; k < Nk; ++k)
                FORGE_TRY(project_k_c3(x, k, c.nLower - 1, &x->h_bph[k * 4], c.bulk.as<double2>()));
        x->have_solve = true;
        x->have_sort = false;
        x->bulk_is_fused = !with_projector;
        return 0;
    }
    for (int64_t k0 = kb; k0 < ke; k0 += B) {
        const int64_t nb = (ke - k0 < B) ? ke - k0 : B;
        FORGE_TRY(launch_assemble(c, c.V.as<double>(), c.P.as<double2>(), k0, nb, c.H.as<double2>()));
        FORGE_TRY(eig_batch_run(x, k0, nb, info));
        if (with_projector)
            for (int64_t k = k0; k < k0 + nb; ++k)
                FORGE_TRY(project_k(x, k, c.nLower - 1, &x->h_bph[k * 4], c.bulk.as<double2>()));
    }
    x->have_solve = true;
    x->have_sort = false;
    x->bulk_is_fused = !with_projector;
    return 0;
}

// P_new = (sum over k of the projector onto bands 1..nLower-1 plus the fully occupied window bands
// of k, plus the partially occupied states with weight zdeg) / Nk: the sum Main.f90:506-511
// forms as GetFock + zFockBulk, with the weight-1 window states folded into each k's product.
int project_fused_once(forge_ctx* x);

// P_new from the solved bands; a bounded tensor-core wait that gave up (FORGE_ERR_TIMEOUT) leaves
// the eigenvectors untouched, and P_new is formed again once
int project_fused(forge_ctx* x) {
    int rc = project_fused_once(x);
    if (rc == FORGE_ERR_TIMEOUT) {
        std::fprintf(stderr, "forge: %s; forming P_new again\n", forge_gpu_last_error());
        rc = project_fused_once(x);
    }
    return rc;
}

int project_fused_once(forge_ctx* x) {
    Context& c = x->c;
    const int64_t N = c.N, Nk = c.Nk;
    const size_t NN = (size_t)N * N;
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    const int64_t nocc = h.nOcc, npart = h.nPart;
    std::vector<WinState> st(nocc > 0 ? nocc : 1);
    if (nocc > 0)
        FORGE_CUDA(cudaMemcpyAsync(st.data(), x->states.ptr, nocc * sizeof(WinState), cudaMemcpyDeviceToHost,
                                   c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    std::vector<int64_t> fk(Nk, 0);
    for (int64_t q = 0; q < nocc - npart; ++q) fk[st[q].k] += 1;
    FORGE_TRY(x->Pn.ensure(4 * NN * sizeof(double2)));
    FORGE_CUDA(cudaMemsetAsync(x->Pn.ptr, 0, 4 * NN * sizeof(double2), c.stream));
    if (x->tcerr.ptr) FORGE_CUDA(cudaMemsetAsync(x->tcerr.ptr, 0, sizeof(int), c.stream));
    const int64_t kb = x->k_begin, ke = (x->k_end > 0) ? x->k_end : Nk;
    for (int64_t k = kb; k < ke; ++k)
        FORGE_TRY(project_k_c3(x, k, c.nLower - 1 + fk[k], &x->h_bph[k * 4], x->Pn.as<double2>()));
    // partially occupied states of local k points (complex weight zdeg in reference mode)
    std::vector<WinState> part;
    for (int64_t q = nocc - npart; q < nocc; ++q)
        if (st[q].k >= kb && st[q].k < ke) part.push_back(st[q]);
    expand_c3_states(x, part);
    if (!part.empty()) {
        // the partial states go to their own buffer: x->states keeps the sorted list (a second
        // formation of P_new reads it again)
        FORGE_TRY(x->pstates.ensure(part.size() * sizeof(WinState)));
        FORGE_CUDA(cudaMemcpyAsync(x->pstates.ptr, part.data(), part.size() * sizeof(WinState),
                                   cudaMemcpyHostToDevice, c.stream));
        FORGE_TRY(window_projector_fp64(c.stream, x->pstates.as<WinState>(), (int64_t)part.size(), c.X.as<double2>(),
                                        c.N, c.N * c.nUpper, c.N, x->Pn.as<double2>()));
    }
    FORGE_CUDA(cudaMemsetAsync(c.bulk.ptr, 0, 4 * NN * sizeof(double2), c.stream));
    FORGE_TRY(scf_combine(c, x->Pn.as<double2>(), c.bulk.as<double2>()));
    if (x->tcerr.ptr) {
        int herr = 0;
        FORGE_CUDA(cudaMemcpyAsync(&herr, x->tcerr.ptr, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        FORGE_CUDA(cudaStreamSynchronize(c.stream));
        if (herr) {
            set_error(FORGE_ERR_TIMEOUT, "tcgen05 projector: a bounded mbarrier wait gave up");
            return FORGE_ERR_TIMEOUT;
        }
    }
    x->have_pnew = true;
    return 0;
}

// ValleyTransform (TightBinding.f90:162-208) of every k's window: Xv = X_win sign(X_win^H V(k) X_win)
int valley_transform_device(forge_ctx* x) {
    Context& c = x->c;
    const int64_t N = c.N, iu = c.nUpper, c0 = c.nLower - 1, nb = c.numb, Nk = c.Nk;
    FORGE_TRY(x->v_W.ensure((size_t)Nk * N * nb * sizeof(double2)));
    FORGE_TRY(x->v_Xv.ensure((size_t)Nk * N * nb * sizeof(double2)));
    FORGE_TRY(x->v_G.ensure((size_t)Nk * nb * nb * sizeof(double2)));
    FORGE_TRY(x->v_S.ensure((size_t)Nk * nb * nb * sizeof(double2)));
    FORGE_TRY(launch_valley_gram(c.stream, c.X.as<double2>(), N, iu, c0, nb, Nk, x->v_rowp.as<int64_t>(),
                                 x->v_col.as<int64_t>(), x->v_coef.as<double>(), x->v_code.as<int>(),
                                 x->v_ph.as<double2>(), x->v_W.as<double2>(), x->v_G.as<double2>()));
    const size_t nn = (size_t)nb * nb;
    std::vector<double2> G(Nk * nn), S(Nk * nn), I(nn, make_double2(0.0, 0.0)), U(nn), Gh(nn);
    std::vector<double> th(nb);
    for (int64_t a = 0; a < nb; ++a) I[a + a * nb] = make_double2(1.0, 0.0);
    FORGE_CUDA(cudaMemcpyAsync(G.data(), x->v_G.ptr, G.size() * sizeof(double2), cudaMemcpyDeviceToHost, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    for (int64_t k = 0; k < Nk; ++k) {
        // unitarize (LapackRoutines.f90:865-893): S = U sign(theta) U^H of the Hermitian part of G
        const double2* g = G.data() + k * nn;
        for (int64_t a = 0; a < nb; ++a)
            for (int64_t b = 0; b < nb; ++b)
                Gh[a + b * nb] = cscale(cadd(g[a + b * nb], cconj(g[b + a * nb])), 0.5);
        if (rr_small((int)nb, Gh.data(), I.data(), th.data(), U.data())) {
            set_error(FORGE_ERR_CUDA, "valley projection: the %lldx%lld eigen-problem failed", (long long)nb,
                      (long long)nb);
            return FORGE_ERR_CUDA;
        }
        double2* sk = S.data() + k * nn;
        for (int64_t a = 0; a < nb; ++a)
            for (int64_t b = 0; b < nb; ++b) {
                double2 acc = make_double2(0.0, 0.0);
                for (int64_t q = 0; q < nb; ++q)
                    acc = cadd(acc, cscale(cmul(U[a + q * nb], cconj(U[b + q * nb])), std::copysign(1.0, th[q])));
                sk[a + b * nb] = acc;
            }
    }
    FORGE_CUDA(cudaMemcpyAsync(x->v_S.ptr, S.data(), S.size() * sizeof(double2), cudaMemcpyHostToDevice, c.stream));
    FORGE_TRY(launch_valley_rotate(c.stream, c.X.as<double2>(), N, iu, c0, nb, Nk, x->v_S.as<double2>(),
                                   x->v_Xv.as<double2>()));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

// Main.f90:470-500: Pn += (GetFock over the window states + GetFock over their valley transforms) / 2;
// st holds every occupied window state with its weighted phases
int valley_window(forge_ctx* x, const std::vector<WinState>& st) {
    Context& c = x->c;
    if (st.empty()) return 0;
    FORGE_TRY(valley_transform_device(x));
    const int64_t n = (int64_t)st.size(), c0 = c.nLower - 1;
    std::vector<WinState> h(st), v(st);
    for (int64_t q = 0; q < n; ++q) {
        for (int t = 0; t < 4; ++t) h[q].wph[t] = v[q].wph[t] = cscale(st[q].wph[t], 0.5);
        v[q].col = st[q].col - c0;
    }
    FORGE_TRY(x->pstates.ensure(n * sizeof(WinState)));
    FORGE_TRY(x->v_st.ensure(n * sizeof(WinState)));
    FORGE_CUDA(cudaMemcpyAsync(x->pstates.ptr, h.data(), n * sizeof(WinState), cudaMemcpyHostToDevice, c.stream));
    FORGE_CUDA(cudaMemcpyAsync(x->v_st.ptr, v.data(), n * sizeof(WinState), cudaMemcpyHostToDevice, c.stream));
    FORGE_TRY(window_projector_fp64(c.stream, x->pstates.as<WinState>(), n, c.X.as<double2>(), c.N, c.N * c.nUpper, c.N,
                                    x->Pn.as<double2>()));
    FORGE_TRY(window_projector_fp64(c.stream, x->v_st.as<WinState>(), n, x->v_Xv.as<double2>(), c.N, c.N * c.numb,
                                    c.N, x->Pn.as<double2>()));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

// P_new with the valley average, for the fused iteration: the bulk bands of every k, then the
// averaged window of Main.f90:470-500, divided by Nk
int project_valley_once(forge_ctx* x) {
    Context& c = x->c;
    const int64_t N = c.N, Nk = c.Nk;
    const size_t NN = (size_t)N * N;
    if (x->k_begin != 0 || (x->k_end > 0 && x->k_end != Nk)) {
        set_error(FORGE_ERR_STATE, "the valley projection runs over the whole k grid (no k shard)");
        return FORGE_ERR_STATE;
    }
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    const int64_t nocc = h.nOcc;
    std::vector<WinState> st(nocc > 0 ? nocc : 0);
    if (nocc > 0)
        FORGE_CUDA(cudaMemcpyAsync(st.data(), x->states.ptr, nocc * sizeof(WinState), cudaMemcpyDeviceToHost,
                                   c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    FORGE_TRY(x->Pn.ensure(4 * NN * sizeof(double2)));
    FORGE_CUDA(cudaMemsetAsync(x->Pn.ptr, 0, 4 * NN * sizeof(double2), c.stream));
    if (x->tcerr.ptr) FORGE_CUDA(cudaMemsetAsync(x->tcerr.ptr, 0, sizeof(int), c.stream));
    for (int64_t k = 0; k < Nk; ++k)
        FORGE_TRY(project_k(x, k, c.nLower - 1, &x->h_bph[k * 4], x->Pn.as<double2>()));
    FORGE_TRY(valley_window(x, st));
    FORGE_CUDA(cudaMemsetAsync(c.bulk.ptr, 0, 4 * NN * sizeof(double2), c.stream));
    FORGE_TRY(scf_combine(c, x->Pn.as<double2>(), c.bulk.as<double2>()));
    if (x->tcerr.ptr) {
        int herr = 0;
        FORGE_CUDA(cudaMemcpyAsync(&herr, x->tcerr.ptr, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        FORGE_CUDA(cudaStreamSynchronize(c.stream));
        if (herr) {
            set_error(FORGE_ERR_TIMEOUT, "tcgen05 projector: a bounded mbarrier wait gave up");
            return FORGE_ERR_TIMEOUT;
        }
    }
    x->have_pnew = true;
    return 0;
}

int project_valley(forge_ctx* x) {
    int rc = project_valley_once(x);
    if (rc == FORGE_ERR_TIMEOUT) {
        std::fprintf(stderr, "forge: %s; forming P_new again\n", forge_gpu_last_error());
        rc = project_valley_once(x);
    }
    return rc;
}

// Main.f90:513-534 on P_new: time reversal, C2, C2T as switched on
int symmetrize_pnew(forge_ctx* x) {
    if (!(x->sym_T || x->sym_C2 || x->sym_C2T)) return 0;
    Context& c = x->c;
    if (!x->have_pnew) {
        set_error(FORGE_ERR_STATE, "symmetrize needs a new density matrix (get_fock) first");
        return FORGE_ERR_STATE;
    }
    FORGE_TRY(x->win.ensure(4 * (size_t)c.N * c.N * sizeof(double2)));
    return launch_symmetrize(c.stream, x->Pn.as<double2>(), x->win.as<double2>(), x->c2_perm.as<int64_t>(), c.N,
                             x->sym_T, x->sym_C2, x->sym_C2T);
}

// forget the mixing history (new state, new precision)
void diis_reset(forge_ctx* x) {
    x->diis_order.clear();
    x->diis_pending = -1;
    x->diis_has_prev = false;
}

// small dense solve G g = b (k <= DIIS_MAX), Gaussian elimination with partial pivoting
bool diis_solve(int k, double G[DIIS_MAX][DIIS_MAX], const double* b, double* g) {
    double A[DIIS_MAX][DIIS_MAX + 1];
    for (int i = 0; i < k; ++i) {
        for (int j = 0; j < k; ++j) A[i][j] = G[i][j];
        A[i][k] = b[i];
    }
    for (int c = 0; c < k; ++c) {
        int piv = c;
        for (int r = c + 1; r < k; ++r)
            if (std::fabs(A[r][c]) > std::fabs(A[piv][c])) piv = r;
        if (A[piv][c] == 0.0) return false;
        if (piv != c)
            for (int j = 0; j <= k; ++j) std::swap(A[c][j], A[piv][j]);
        for (int r = c + 1; r < k; ++r) {
            const double f = A[r][c] / A[c][c];
            for (int j = c; j <= k; ++j) A[r][j] -= f * A[c][j];
        }
    }
    for (int i = k - 1; i >= 0; --i) {
        double t = A[i][k];
        for (int j = i + 1; j < k; ++j) t -= A[i][j] * g[j];
        g[i] = t / A[i][i];
    }
    return true;
}

// Anderson / Pulay step: x_next = x + beta r - sum_i g_i (dX_i + beta dR_i), with g minimising
// |r - sum_i g_i dR_i| over the last `depth` (dX, dR) pairs.  c.P holds x, x->Pn holds P_new.
int pulay_step(forge_ctx* x) {
    Context& c = x->c;
    const size_t nn4 = 4 * (size_t)c.N * c.N;
    if (x->diis_nslots == 0) {
        // as many slots as memory allows, up to depth + 1 (each slot: dX and dR, complex64)
        size_t freeb = 0, totalb = 0;
        cudaMemGetInfo(&freeb, &totalb);
        const size_t slot = 2 * nn4 * sizeof(float2);
        const size_t avail = freeb > ((size_t)6 << 30) + nn4 * sizeof(float2) ? freeb - ((size_t)6 << 30) - nn4 * sizeof(float2) : 0;
        int ns = std::min<int>(x->diis_depth + 1, DIIS_MAX);
        while (ns > 2 && (size_t)ns * slot > avail) --ns;
        FORGE_TRY(x->diis_hist.ensure((size_t)ns * slot));
        FORGE_TRY(x->diis_rprev.ensure(nn4 * sizeof(float2)));
        FORGE_TRY(x->diis_part.ensure(scf_diis_parts() * sizeof(double)));
        x->diis_nslots = ns;
    }
    DiisArgs d{};
    d.P = c.P.as<double2>();
    d.Pn = x->Pn.as<double2>();
    d.hist = x->diis_hist.as<float2>();
    d.rprev = x->diis_rprev.as<float2>();
    d.nn4 = nn4;
    d.beta = x->diis_beta;
    d.part = x->diis_part.as<double>();
    const int depth = x->diis_nslots - 1;
    if (!x->diis_has_prev) {
        // first step: linear mixing; its dX waits in slot 0 for the next residual
        d.nslots = 0;
        d.spend = 0;
        FORGE_TRY(scf_diis_update(c, d));
        x->diis_pending = 0;
        x->diis_has_prev = true;
        x->diis_order.clear();
        return 0;
    }
    // complete the pending pair with dR = r - r_prev; dots with every complete pair
    const int snew = x->diis_pending;
    std::vector<int> list = x->diis_order;
    list.push_back(snew);
    d.snew = snew;
    d.nslots = (int)list.size();
    for (int i = 0; i < d.nslots; ++i) d.slots[i] = list[i];
    FORGE_TRY(scf_diis_dots(c, d));
    std::vector<double> part(scf_diis_parts());
    FORGE_CUDA(cudaMemcpyAsync(part.data(), d.part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    double a[DIIS_MAX] = {}, bv[DIIS_MAX] = {};
    const size_t nparts = part.size() / (2 * DIIS_MAX);
    for (size_t q = 0; q < nparts; ++q)
        for (int i = 0; i < d.nslots; ++i) {
            a[i] += part[q * 2 * DIIS_MAX + i];
            bv[i] += part[q * 2 * DIIS_MAX + DIIS_MAX + i];
        }
    for (int i = 0; i < d.nslots; ++i) {
        x->diis_G[list[i]][snew] = a[i];
        x->diis_G[snew][list[i]] = a[i];
    }
    double bmap[DIIS_MAX] = {};
    for (int i = 0; i < d.nslots; ++i) bmap[list[i]] = bv[i];
    x->diis_order.push_back(snew);
    // keep `depth` complete pairs; the evicted slot takes the next dX
    int spend;
    if ((int)x->diis_order.size() > depth) {
        spend = x->diis_order.front();
        x->diis_order.erase(x->diis_order.begin());
    } else {
        spend = -1;
        for (int sl = 0; sl < x->diis_nslots && spend < 0; ++sl)
            if (std::find(x->diis_order.begin(), x->diis_order.end(), sl) == x->diis_order.end()) spend = sl;
    }
    // least squares on the complete pairs, lightly regularised
    const int k = (int)x->diis_order.size();
    double G[DIIS_MAX][DIIS_MAX], b[DIIS_MAX], g[DIIS_MAX] = {};
    double gmax = 0.0;
    for (int i = 0; i < k; ++i) gmax = std::max(gmax, x->diis_G[x->diis_order[i]][x->diis_order[i]]);
    for (int i = 0; i < k; ++i) {
        for (int j = 0; j < k; ++j) G[i][j] = x->diis_G[x->diis_order[i]][x->diis_order[j]];
        G[i][i] += 1e-10 * gmax;
        b[i] = bmap[x->diis_order[i]];
    }
    if (!diis_solve(k, G, b, g))
        for (int i = 0; i < k; ++i) g[i] = 0.0;
    d.nslots = k;
    for (int i = 0; i < k; ++i) {
        d.slots[i] = x->diis_order[i];
        d.gamma[i] = g[i];
    }
    d.spend = spend;
    FORGE_TRY(scf_diis_update(c, d));
    x->diis_pending = spend;
    return 0;
}

int sort_device(forge_ctx* x, double nfilling) {
    Context& c = x->c;
    if (!x->have_solve) {
        set_error(FORGE_ERR_STATE, "sort before solve");
        return FORGE_ERR_STATE;
    }
    const int64_t nw = c.numb * c.Nk;
    FORGE_TRY(x->sorted_e.ensure(nw * sizeof(double)));
    FORGE_TRY(x->sorted_idx.ensure(nw * sizeof(int64_t)));
    FORGE_TRY(x->states.ensure(nw * sizeof(WinState)));
    FORGE_TRY(launch_sort_fermi(c, x->w.as<double>(), nfilling, x->sorted_e.as<double>(), x->sorted_idx.as<int64_t>(),
                                x->states.as<WinState>(), x->sc.as<ScfScalars>()));
    x->have_sort = true;
    return 0;
}

// the bulk projector of bands 1..nLower-1 when the last solve left it out (the fused SCF iteration
// and the group solve fold it into P_new instead)
int ensure_bulk(forge_ctx* x) {
    if (!x->bulk_is_fused) return 0;
    Context& c = x->c;
    FORGE_TRY(c.bulk.ensure(4 * (size_t)c.N * c.N * sizeof(double2)));
    FORGE_CUDA(cudaMemsetAsync(c.bulk.ptr, 0, 4 * (size_t)c.N * c.N * sizeof(double2), c.stream));
    if (x->tcerr.ptr) FORGE_CUDA(cudaMemsetAsync(x->tcerr.ptr, 0, sizeof(int), c.stream));
    const int64_t kb = x->k_begin, ke = (x->k_end > 0) ? x->k_end : c.Nk;
    for (int64_t k = kb; k < ke; ++k)
        FORGE_TRY(project_k_c3(x, k, c.nLower - 1, &x->h_bph[k * 4], c.bulk.as<double2>()));
    x->bulk_is_fused = false;
    return 0;
}

int get_fock_device(forge_ctx* x, int64_t nstates) {
    Context& c = x->c;
    FORGE_TRY(ensure_bulk(x));
    const size_t NN = (size_t)c.N * c.N;
    FORGE_TRY(x->Pn.ensure(4 * NN * sizeof(double2)));
    FORGE_CUDA(cudaMemsetAsync(x->Pn.ptr, 0, 4 * NN * sizeof(double2), c.stream));
    FORGE_TRY(window_projector_fp64(c.stream, x->states.as<WinState>(), nstates, c.X.as<double2>(), c.N,
                                    c.N * c.nUpper, c.N, x->Pn.as<double2>()));
    FORGE_TRY(scf_combine(c, x->Pn.as<double2>(), c.bulk.as<double2>()));
    x->have_pnew = true;
    return 0;
}

int read_scalars(forge_ctx* x, ScfScalars* h) {
    Context& c = x->c;
    FORGE_CUDA(cudaMemcpyAsync(h, x->sc.ptr, sizeof(ScfScalars), cudaMemcpyDeviceToHost, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

int write_scalars(forge_ctx* x, const ScfScalars* h) {
    Context& c = x->c;
    FORGE_CUDA(cudaMemcpyAsync(x->sc.ptr, h, sizeof(ScfScalars), cudaMemcpyHostToDevice, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

// energies and potential of the current state P (Main.f90:290-346)
int prepare_state_device(forge_ctx* x, double* Energies) {
    Context& c = x->c;
    FORGE_TRY(scf_density(c, c.P.as<double2>(), c.dens.as<double>()));
    FORGE_TRY(scf_energy_forms(c, x->te.as<double>(), c.P.as<double2>(), c.P.as<double2>(), c.dens.as<double>(),
                               c.dens.as<double>(), x->y.as<double>(), x->work.as<double>(), x->sc.as<ScfScalars>()));
    FORGE_TRY(scf_oda(c, x->sc.as<ScfScalars>(), 1));
    FORGE_TRY(scf_potential(c, x->y.as<double>(), c.dens.as<double>(), c.V.as<double>()));
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    for (int t = 0; t < 4; ++t) h.Ein[t] = h.Eout[t];
    FORGE_TRY(write_scalars(x, &h));
    if (Energies)
        for (int t = 0; t < 4; ++t) Energies[t] = h.Eout[t];
    x->have_state = true;
    return 0;
}

// Anderson / Pulay mixing of (P_in, P_new) after the energy-forms pass of the pair: the residual,
// the mixed state, its density, potential and energies
int pulay_mix(forge_ctx* x) {
    Context& c = x->c;
    ScfScalars* sc = x->sc.as<ScfScalars>();
    FORGE_TRY(scf_diis_residual(c, x->y.as<double>(), c.dens.as<double>(), x->dens_new.as<double>(),
                                x->work.as<double>(), sc));
    FORGE_TRY(pulay_step(x));
    FORGE_TRY(scf_diis_dens(c, c.P.as<double2>(), c.dens.as<double>(), x->work.as<double>(), sc));
    FORGE_TRY(scf_energy_forms(c, x->te.as<double>(), c.P.as<double2>(), c.P.as<double2>(), c.dens.as<double>(),
                               c.dens.as<double>(), x->y.as<double>(), x->work.as<double>(), sc));
    FORGE_TRY(scf_potential(c, x->y.as<double>(), c.dens.as<double>(), c.V.as<double>()));
    FORGE_TRY(scf_oda(c, sc, 1));
    return scf_diis_commit(c, sc);
}

// One batched eigen-solve over the H(k) of every k of several contexts of different ndim (the
// uneven-size batch): each H(k) is assembled by its own context into a scratch matrix, embedded in
// an nmax x nmax slot (launch_pad_slot), the slots are solved in batches by the context precision's
// solver (zdiagRed, iu = the largest nUpper), the mixed path's FP64 window Rayleigh-Ritz runs per
// slot on that system's own window, and each context receives its eigenpairs 1..nUpper.  All
// work runs on the first context's stream.
int solve_group_device(forge_ctx** xs, int64_t nctx, int* infos) {
    forge_ctx* x0 = xs[0];
    Context& c0 = x0->c;
    cudaStream_t st = c0.stream;
    int64_t nmax = 0, iumax = 0;
    std::vector<std::pair<int64_t, int64_t>> items;
    for (int64_t b = 0; b < nctx; ++b) {
        forge_ctx* x = xs[b];
        Context& c = x->c;
        if (c.precision != c0.precision || x->c3 || x->valley || x->k_begin != 0 || x->k_end != 0 || x->oa_mode != 0) {
            set_error(FORGE_ERR_ARG, "solve_group: context %lld differs in precision or uses C3, valley, k shards or "
                      "the eigenpair refinement (not available in a group)", (long long)b);
            return FORGE_ERR_ARG;
        }
        if (!c.lr_ready) FORGE_TRY(launch_long_range(c));
        nmax = std::max<int64_t>(nmax, c.N);
        iumax = std::max<int64_t>(iumax, c.nUpper);
        for (int64_t k = 0; k < c.Nk; ++k) items.push_back({b, k});
        FORGE_TRY(c.X.ensure((size_t)c.Nk * c.N * c.nUpper * sizeof(double2)));
        FORGE_TRY(x->w.ensure((size_t)c.Nk * c.nUpper * sizeof(double)));
        FORGE_TRY(c.bulk.ensure(4 * (size_t)c.N * c.N * sizeof(double2)));
        infos[b] = 0;
    }
    const bool mixed = c0.precision == FORGE_PREC_MIXED;
    const size_t slot = (size_t)nmax * nmax;
    size_t per_item = slot * 16 + eig_workspace_bytes(nmax, iumax, 1) + (size_t)nmax * iumax * 16 + iumax * 8;
    if (mixed) per_item += eig_mixed_workspace_bytes(nmax, iumax, 1);
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    const size_t reserve = ((size_t)8 << 30) + slot * 16;
    int64_t B = (int64_t)((freeb > reserve ? freeb - reserve : freeb / 4) / per_item);
    B = std::max<int64_t>(1, std::min<int64_t>(B, (int64_t)items.size()));
    FORGE_TRY(x0->g_H.ensure((size_t)B * slot * sizeof(double2)));
    FORGE_TRY(x0->g_X.ensure((size_t)B * nmax * iumax * sizeof(double2)));
    FORGE_TRY(x0->g_w.ensure((size_t)B * iumax * sizeof(double)));
    FORGE_TRY(x0->g_eigws.ensure(eig_workspace_bytes(nmax, iumax, B)));
    if (mixed) FORGE_TRY(x0->g_mixws.ensure(eig_mixed_workspace_bytes(nmax, iumax, B)));
    FORGE_TRY(x0->g_tmp.ensure(slot * sizeof(double2)));
    FORGE_TRY(x0->g_rows.ensure(nmax * sizeof(double)));
    FORGE_TRY(x0->g_sig.ensure(sizeof(double)));
    if (mixed && x0->rr_width > 0) FORGE_TRY(x0->g_rr.ensure(rr_window_workspace_bytes(nmax, 1)));
    double2* gH = x0->g_H.as<double2>();
    double2* gX = x0->g_X.as<double2>();
    double* gw = x0->g_w.as<double>();
    for (size_t q0 = 0; q0 < items.size(); q0 += (size_t)B) {
        const int64_t nb = std::min<int64_t>(B, (int64_t)(items.size() - q0));
        for (int64_t q = 0; q < nb; ++q) {
            Context& cb = xs[items[q0 + q].first]->c;
            const cudaStream_t own = cb.stream;
            cb.stream = st;   // the assembly of every member on the group's stream
            const int rc = launch_assemble(cb, cb.V.as<double>(), cb.P.as<double2>(), items[q0 + q].second, 1,
                                           x0->g_tmp.as<double2>());
            cb.stream = own;
            FORGE_TRY(rc);
            FORGE_TRY(launch_pad_slot(st, x0->g_tmp.as<double2>(), cb.N, gH + q * slot, nmax, x0->g_rows.as<double>(),
                                      x0->g_sig.as<double>()));
        }
        EigArgs g{};
        g.n = nmax;
        g.iu = iumax;
        g.batch = nb;
        g.A = gH;
        g.lda = nmax;
        g.strideA = (int64_t)slot;
        g.X = gX;
        g.ldx = nmax;
        g.strideX = nmax * iumax;
        g.w = gw;
        g.ortol_rel = 1e-7;
        eig_bind_workspace(g, x0->g_eigws.ptr);
        FORGE_TRY(mixed ? eig_mixed(st, g, x0->g_mixws.ptr) : eig_fp64(st, g));
        if (mixed && x0->rr_width > 0)
            for (int64_t q = 0; q < nb; ++q) {
                const int64_t iub = xs[items[q0 + q].first]->c.nUpper;
                const int64_t nw = std::min<int64_t>(x0->rr_width, iub);
                FORGE_TRY(rr_window(st, gH + q * slot, (int64_t)slot, gX + q * nmax * iumax, nmax, nmax * iumax,
                                    gw + q * iumax, iumax, nmax, iub - nw, nw, 1, x0->g_rr.ptr));
            }
        std::vector<int> fails(nb);
        FORGE_CUDA(cudaMemcpyAsync(fails.data(), g.fail, nb * sizeof(int), cudaMemcpyDeviceToHost, st));
        for (int64_t q = 0; q < nb; ++q) {
            const int64_t b = items[q0 + q].first, k = items[q0 + q].second;
            Context& cb = xs[b]->c;
            const int64_t Nb = cb.N, iub = cb.nUpper;
            FORGE_CUDA(cudaMemcpy2DAsync(cb.X.as<double2>() + (size_t)k * Nb * iub, Nb * sizeof(double2),
                                         gX + q * nmax * iumax, nmax * sizeof(double2), Nb * sizeof(double2), iub,
                                         cudaMemcpyDeviceToDevice, st));
            FORGE_CUDA(cudaMemcpyAsync(xs[b]->w.as<double>() + (size_t)k * iub, gw + q * iumax, iub * sizeof(double),
                                       cudaMemcpyDeviceToDevice, st));
        }
        FORGE_CUDA(cudaStreamSynchronize(st));
        for (int64_t q = 0; q < nb; ++q) infos[items[q0 + q].first] += fails[q] ? 1 : 0;
    }
    for (int64_t b = 0; b < nctx; ++b) {
        forge_ctx* x = xs[b];
        Context& c = x->c;
        x->h_bph.resize(c.Nk * 4);
        FORGE_CUDA(cudaMemcpy(x->h_bph.data(), c.bphase.ptr, c.Nk * 4 * sizeof(double2), cudaMemcpyDeviceToHost));
        x->oa_active = false;
        c.refined = false;
        x->have_solve = true;
        x->have_sort = false;
        x->bulk_is_fused = true;
    }
    return 0;
}

// forge_gpu_scf_iteration before its solve: checks, the input energies into the device scalars
int scf_iteration_begin(forge_ctx* x, double* Energies, double* Ein) {
    Context& c = x->c;
    if (!x->have_state) {
        set_error(FORGE_ERR_STATE, "scf_iteration needs plain_guess or set_state + prepare_state first");
        return FORGE_ERR_STATE;
    }
    if (!c.lr_ready) FORGE_TRY(launch_long_range(c));
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    if (Energies) {
        for (int t = 0; t < 4; ++t) h.Ein[t] = Energies[t];
        FORGE_TRY(write_scalars(x, &h));
    }
    for (int t = 0; t < 4; ++t) Ein[t] = h.Ein[t];
    return 0;
}

// forge_gpu_scf_iteration after its solve (eigenpairs of every k in c.X / w): sort, Fermi level,
// P_new, energies, mixing and potential (Main.f90:392-595), and the report
int scf_iteration_end(forge_ctx* x, const double* Ein, int info, double* Energies, forge_iter_report* rep) {
    Context& c = x->c;
    FORGE_TRY(sort_device(x, c.s.nfilling));
    FORGE_TRY(x->valley ? project_valley(x) : project_fused(x));
    FORGE_TRY(symmetrize_pnew(x));
    FORGE_TRY(scf_density(c, x->Pn.as<double2>(), x->dens_new.as<double>()));
    FORGE_TRY(scf_energy_forms(c, x->te.as<double>(), c.P.as<double2>(), x->Pn.as<double2>(), c.dens.as<double>(),
                               x->dens_new.as<double>(), x->y.as<double>(), x->work.as<double>(),
                               x->sc.as<ScfScalars>()));
    if (x->mix_mode == FORGE_MIX_PULAY) {
        FORGE_TRY(pulay_mix(x));
    } else {
        FORGE_TRY(scf_oda(c, x->sc.as<ScfScalars>(), x->mix_mode == FORGE_MIX_LINEAR ? 2 : 0, x->diis_beta));
        FORGE_TRY(scf_mix(c, c.P.as<double2>(), x->Pn.as<double2>(), c.dens.as<double>(), c.V.as<double>(),
                          x->y.as<double>(), x->work.as<double>(), x->sc.as<ScfScalars>()));
    }
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    x->have_pnew = false;
    x->last_residual = h.residual;
    if (Energies)
        for (int t = 0; t < 4; ++t) Energies[t] = h.Eout[t];
    if (rep) {
        rep->refined = x->oa_active ? 1 : 0;
        rep->Step = h.step;
        rep->DensityConvergence = h.dn_max;
        rep->TotalEnergyIn = h.Etot_in;
        rep->TotalEnergy = h.Etot_out;
        rep->KineticEnergyIn = Ein[0];
        rep->FockEnergyIn = Ein[1];
        rep->HartreeEnergyIn = Ein[2];
        rep->HubbardEnergyIn = Ein[3];
        rep->KineticEnergy = h.Eout[0];
        rep->FockEnergy = h.Eout[1];
        rep->HartreeEnergy = h.Eout[2];
        rep->HubbardEnergy = h.Eout[3];
        rep->FermiEnergy = h.EF;
        rep->DegFactor = h.DegFactor;
        rep->residual = h.residual;
        rep->nFermiLevel = h.nF;
        rep->nOccStates = h.nOcc;
        rep->nPartOccStates = h.nPart;
        rep->info = info;
    }
    return 0;
}

}  // namespace

extern "C" {

const char* forge_gpu_last_error(void) { return g_err.c_str(); }
int64_t forge_gpu_launch_count(void) { return g_launches.load(); }
int forge_gpu_version(void) { return 1; }

int forge_gpu_init(const forge_setup* s, const double* Coords, const int64_t* nUnitCell_1, const int64_t* nUnitCell_2,
                   const double* tn, const double* MomentaValues, const int64_t* nMomentaComponents,
                   forge_ctx** out) {
    if (!s || !Coords || !nUnitCell_1 || !nUnitCell_2 || !tn || !MomentaValues || !nMomentaComponents || !out) {
        set_error(FORGE_ERR_ARG, "forge_gpu_init: null argument");
        return FORGE_ERR_ARG;
    }
    *out = nullptr;
    if (s->numS != 1) {
        set_error(FORGE_ERR_ARG, "numS=%lld is not supported (only numS=1)", (long long)s->numS);
        return FORGE_ERR_ARG;
    }
    if (s->fphase != 0) {
        // the projectors apply no site phase exp(i vk.r fphase) (HartreeFock.f90:453, 514)
        set_error(FORGE_ERR_ARG, "fphase=%lld is not supported (only fphase=0)", (long long)s->fphase);
        return FORGE_ERR_ARG;
    }
    if (s->numNeighborCells != 4) {
        set_error(FORGE_ERR_ARG, "numNeighborCells=%lld is not supported (numI=1 gives 4)",
                  (long long)s->numNeighborCells);
        return FORGE_ERR_ARG;
    }
    const int64_t nexp = s->nlayers * 2 * (s->ntheta * s->ntheta + (s->ntheta + 1) * (s->ntheta + 1) +
                                           (s->ntheta + 1) * s->ntheta);
    if (s->ndim != nexp || s->ndim < 2 || s->numk < 1 || s->nUpper > s->ndim || s->nLower < 1 ||
        s->nUpper - s->nLower + 1 != s->numb) {
        set_error(FORGE_ERR_ARG, "inconsistent setup (ndim=%lld expected %lld, nLower=%lld nUpper=%lld numb=%lld)",
                  (long long)s->ndim, (long long)nexp, (long long)s->nLower, (long long)s->nUpper,
                  (long long)s->numb);
        return FORGE_ERR_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        set_error(FORGE_ERR_CUDA, "no CUDA device");
        return FORGE_ERR_CUDA;
    }
    forge_ctx* x = new forge_ctx();
    Context& c = x->c;
    c.s = *s;
    c.N = s->ndim;
    c.Nk = s->numk * s->numk;
    c.nnc = 4;
    c.nLower = s->nLower;
    c.nUpper = s->nUpper;
    c.numb = s->numb;
    c.NP = s->NeutralityPoint;
    c.precision = (int)s->precision;
    c.t1[0] = tn[0];
    c.t1[1] = tn[1];
    c.t2[0] = tn[2];
    c.t2[1] = tn[3];
    c.ucell1.assign(nUnitCell_1, nUnitCell_1 + 4);
    c.ucell2.assign(nUnitCell_2, nUnitCell_2 + 4);
    c.kcomp.assign(nMomentaComponents, nMomentaComponents + 2 * c.Nk);
    c.kvals.assign(MomentaValues, MomentaValues + 2 * s->numk * s->numk);
    c.coords_h.assign(Coords, Coords + 3 * c.N);
    int rc = 0;
    auto fail = [&](int r) {
        forge_gpu_finalize(x);
        return r;
    };
    if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_error(FORGE_ERR_CUDA, "stream creation failed");
        delete x;
        return FORGE_ERR_CUDA;
    }
    x->prof.stream = c.stream;
    set_current_profiler(&x->prof);
    const int64_t N = c.N, Nk = c.Nk, numk = s->numk;
    // phases: exp(-i k.R_c) with the floating-point dot (HartreeFock.f90:90) and the integer
    // Bloch phase exp(-2 pi i (ivk1 n1 + ivk2 n1 + ivk2 n2)/numk) (HartreeFock.f90:471)
    std::vector<double2> kph(Nk * 3), bph(Nk * 4);
    std::vector<double> kvec(Nk * 2);
    const double pi = 4.0 * std::atan(1.0);
    for (int64_t k = 0; k < Nk; ++k) {
        const int64_t ivk1 = c.kcomp[k], ivk2 = c.kcomp[k + Nk];
        const double vk0 = c.kvals[ivk1 + ivk2 * numk], vk1 = c.kvals[ivk1 + ivk2 * numk + numk * numk];
        kvec[2 * k] = vk0;
        kvec[2 * k + 1] = vk1;
        for (int q = 0; q < 4; ++q) {
            const int64_t n1 = c.ucell1[q], n2 = c.ucell2[q];
            if (q > 0) {
                const double rx = (double)n1 * c.t1[0] + (double)n2 * c.t2[0];
                const double ry = (double)n1 * c.t1[1] + (double)n2 * c.t2[1];
                const double th = vk0 * rx + vk1 * ry;
                kph[k * 3 + q - 1] = make_double2(std::cos(th), -std::sin(th));
            }
            const double ph = -(2.0 * pi * (double)(ivk1 * n1 + ivk2 * n1 + ivk2 * n2) / (double)numk);
            bph[k * 4 + q] = (q == 0) ? make_double2(1.0, 0.0) : make_double2(std::cos(ph), std::sin(ph));
        }
    }
    const size_t NN = (size_t)N * N;
    if ((rc = c.coords.ensure(3 * N * sizeof(double))) || (rc = c.kphase.ensure(Nk * 3 * sizeof(double2))) ||
        (rc = c.bphase.ensure(Nk * 4 * sizeof(double2))) || (rc = c.kvecs.ensure(Nk * 2 * sizeof(double))) ||
        (rc = c.P.ensure(4 * NN * sizeof(double2))) || (rc = c.V.ensure(N * sizeof(double))) ||
        (rc = c.dens.ensure(N * sizeof(double))) || (rc = x->dens_new.ensure(N * sizeof(double))) ||
        (rc = x->sc.ensure(sizeof(ScfScalars))) || (rc = x->work.ensure(scf_work_doubles(N) * sizeof(double))) ||
        (rc = x->y.ensure(2 * N * sizeof(double))))
        return fail(rc);
    if (cudaMemcpyAsync(c.coords.ptr, Coords, 3 * N * sizeof(double), cudaMemcpyHostToDevice, c.stream) ||
        cudaMemcpyAsync(c.kphase.ptr, kph.data(), Nk * 3 * sizeof(double2), cudaMemcpyHostToDevice, c.stream) ||
        cudaMemcpyAsync(c.bphase.ptr, bph.data(), Nk * 4 * sizeof(double2), cudaMemcpyHostToDevice, c.stream) ||
        cudaMemcpyAsync(c.kvecs.ptr, kvec.data(), Nk * 2 * sizeof(double), cudaMemcpyHostToDevice, c.stream) ||
        cudaMemsetAsync(c.P.ptr, 0, 4 * NN * sizeof(double2), c.stream) ||
        cudaMemsetAsync(c.V.ptr, 0, N * sizeof(double), c.stream) ||
        cudaMemsetAsync(x->sc.ptr, 0, sizeof(ScfScalars), c.stream)) {
        set_error(FORGE_ERR_CUDA, "forge_gpu_init: upload failed");
        return fail(FORGE_ERR_CUDA);
    }
    if ((rc = launch_pair_tables(c)) || (rc = build_energy_tables(c, x->te))) return fail(rc);
    if (cudaStreamSynchronize(c.stream) != cudaSuccess) {
        set_error(FORGE_ERR_CUDA, "forge_gpu_init: %s", cudaGetErrorString(cudaGetLastError()));
        return fail(FORGE_ERR_CUDA);
    }
    *out = x;
    return 0;
}

int forge_gpu_finalize(forge_ctx* x) {
    if (!x) return 0;
    Context& c = x->c;
    if (c.stream) cudaStreamSynchronize(c.stream);
    x->prof.release();
    if (current_profiler() == &x->prof) set_current_profiler(nullptr);
    for (cudaEvent_t& e : x->marks)
        if (e) cudaEventDestroy(e);
    DevBuf* bufs[] = {&c.coords, &c.tab_t, &c.tab_v, &c.LR, &c.P, &c.P_in, &c.P_new, &c.bulk, &c.V, &c.dens,
                      &c.dens_in, &c.V_old, &c.H, &c.X, &c.bands, &c.evals, &c.kvecs, &c.kphase, &c.bphase,
                      &c.sort_idx, &c.sort_e, &c.red, &c.scalars, &x->te, &x->Pn, &x->win, &x->eigws, &x->mixws,
                      &x->states, &x->sorted_e, &x->sorted_idx, &x->sc, &x->work, &x->y, &x->dens_new, &x->w,
                      &x->projws, &x->tcerr, &x->diis_hist, &x->diis_rprev, &x->diis_part, &x->rrws, &x->pstates,
                      &x->c3_Xr, &x->c3_wr, &x->c3_tab, &x->c3_perm, &x->c3_phase, &x->c2_perm,
                      &x->v_rowp, &x->v_col, &x->v_coef, &x->v_code, &x->v_ph, &x->v_W, &x->v_G, &x->v_S,
                      &x->v_Xv, &x->v_st, &x->oaws, &x->w_all, &x->g_H, &x->g_X, &x->g_w, &x->g_eigws,
                      &x->g_mixws, &x->g_tmp, &x->g_rows, &x->g_sig, &x->g_rr};
    for (DevBuf* b : bufs) b->release();
    if (c.stream) cudaStreamDestroy(c.stream);
    delete x;
    return 0;
}

int forge_gpu_set_precision(forge_ctx* x, int64_t precision) {
    FORGE_TRY(check_ctx(x));
    if (precision != FORGE_PREC_FP64 && precision != FORGE_PREC_MIXED) {
        set_error(FORGE_ERR_ARG, "unknown precision %lld", (long long)precision);
        return FORGE_ERR_ARG;
    }
    if (x->c.precision != (int)precision) {
        x->c.precision = (int)precision;
        x->eig_batch = 0;
        diis_reset(x);   // the residual map changes with the precision
    }
    return 0;
}

int forge_gpu_set_refinement(forge_ctx* x, int64_t width) {
    FORGE_TRY(check_ctx(x));
    if (width < 0 || width > 32) {
        set_error(FORGE_ERR_ARG, "set_refinement: width %lld outside 0..32", (long long)width);
        return FORGE_ERR_ARG;
    }
    x->rr_width = width;
    return 0;
}

int forge_gpu_set_eigen_refinement(forge_ctx* x, int64_t mode, double residual_below, double delta, int64_t depth) {
    FORGE_TRY(check_ctx(x));
    if (mode < 0 || mode > 2 || depth < 0 || depth > 4 || !(residual_below >= 0.0) || !(delta >= 0.0)) {
        set_error(FORGE_ERR_ARG, "set_eigen_refinement: mode 0..2, depth 0..4, residual_below >= 0, delta >= 0");
        return FORGE_ERR_ARG;
    }
    if ((x->oa_mode != 0) != (mode != 0)) x->eig_batch = 0;   // the solve's memory per k changes
    x->oa_mode = (int)mode;
    x->oa_below = residual_below;
    x->oa_delta = delta > 0.0 ? delta : 1e-3;
    x->oa_depth = depth > 0 ? (int)depth : 4;
    return 0;
}

int forge_gpu_last_refined(forge_ctx* x, int64_t* refined) {
    FORGE_TRY(check_ctx(x));
    if (refined) *refined = x->oa_active ? 1 : 0;
    return 0;
}

int forge_gpu_set_c3(forge_ctx* x, int64_t nenforceC3, const int64_t* nC3pairs, const int64_t* RotateLayers) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (nenforceC3 == 0) {
        x->c3 = false;
        x->have_solve = x->have_sort = false;
        return 0;
    }
    if (nenforceC3 != 1 || !nC3pairs || !RotateLayers) {
        set_error(FORGE_ERR_ARG, "set_c3: nenforceC3 must be 0 or 1, with nC3pairs and RotateLayers");
        return FORGE_ERR_ARG;
    }
    if (c.s.fphase != 0) {
        set_error(FORGE_ERR_ARG, "set_c3: the C3-reduced solve is implemented for fphase = 0");
        return FORGE_ERR_ARG;
    }
    if (x->valley) {
        set_error(FORGE_ERR_ARG, "set_c3: the C3-reduced solve is not combined with the valley projection");
        return FORGE_ERR_ARG;
    }
    const int64_t N = c.N;
    // nC3pairs (C3_RelatedPoints, Geometry.f90:1172-1223) must be a permutation of the sites
    std::vector<char> seen(N, 0);
    for (int64_t i = 0; i < N; ++i) {
        const int64_t j = nC3pairs[i];
        if (j < 1 || j > N || seen[j - 1]) {
            set_error(FORGE_ERR_ARG, "set_c3: nC3pairs is not a permutation of 1..%lld (site %lld)", (long long)N,
                      (long long)(i + 1));
            return FORGE_ERR_ARG;
        }
        seen[j - 1] = 1;
    }
    C3Tables t;
    FORGE_TRY(c3_build_tables(c.s.numk, N, c.s.nlayers, c.kcomp.data(), RotateLayers, t));
    std::vector<int64_t> perm(3 * N);
    for (int64_t i = 0; i < N; ++i) {
        perm[i] = i;
        perm[N + i] = nC3pairs[i] - 1;
        perm[2 * N + i] = nC3pairs[nC3pairs[i] - 1] - 1;
    }
    FORGE_TRY(x->c3_tab.ensure(t.slot_tab.size() * sizeof(int64_t)));
    FORGE_TRY(x->c3_perm.ensure(perm.size() * sizeof(int64_t)));
    FORGE_TRY(x->c3_phase.ensure(t.phase.size() * sizeof(double2)));
    FORGE_CUDA(cudaMemcpyAsync(x->c3_tab.ptr, t.slot_tab.data(), t.slot_tab.size() * sizeof(int64_t),
                               cudaMemcpyHostToDevice, c.stream));
    FORGE_CUDA(cudaMemcpyAsync(x->c3_perm.ptr, perm.data(), perm.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                               c.stream));
    FORGE_CUDA(cudaMemcpyAsync(x->c3_phase.ptr, t.phase.data(), t.phase.size() * sizeof(double2),
                               cudaMemcpyHostToDevice, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    x->c3t = std::move(t);
    x->c3 = true;
    x->eig_batch = 0;
    x->have_solve = x->have_sort = false;
    return 0;
}

int forge_gpu_set_valley(forge_ctx* x, int64_t nenforceValley, const int64_t* RotateLayers) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (nenforceValley == 0) {
        x->valley = false;
        return 0;
    }
    if (nenforceValley != 1 || !RotateLayers) {
        set_error(FORGE_ERR_ARG, "set_valley: nenforceValley must be 0 or 1, with RotateLayers");
        return FORGE_ERR_ARG;
    }
    if (x->c3) {
        set_error(FORGE_ERR_ARG, "set_valley: the valley projection is not combined with the C3-reduced solve");
        return FORGE_ERR_ARG;
    }
    ValleyTerms t;
    FORGE_TRY(valley_build_terms(c, RotateLayers, t));
    std::vector<double2> ph;
    valley_phases(c, ph);
    const size_t nnz = t.col.size();
    FORGE_TRY(x->v_rowp.ensure(t.rowp.size() * sizeof(int64_t)));
    FORGE_TRY(x->v_col.ensure((nnz ? nnz : 1) * sizeof(int64_t)));
    FORGE_TRY(x->v_coef.ensure((nnz ? nnz : 1) * sizeof(double)));
    FORGE_TRY(x->v_code.ensure((nnz ? nnz : 1) * sizeof(int)));
    FORGE_TRY(x->v_ph.ensure(ph.size() * sizeof(double2)));
    FORGE_CUDA(cudaMemcpyAsync(x->v_rowp.ptr, t.rowp.data(), t.rowp.size() * sizeof(int64_t), cudaMemcpyHostToDevice,
                               c.stream));
    if (nnz) {
        FORGE_CUDA(cudaMemcpyAsync(x->v_col.ptr, t.col.data(), nnz * sizeof(int64_t), cudaMemcpyHostToDevice, c.stream));
        FORGE_CUDA(cudaMemcpyAsync(x->v_coef.ptr, t.coef.data(), nnz * sizeof(double), cudaMemcpyHostToDevice,
                                   c.stream));
        FORGE_CUDA(cudaMemcpyAsync(x->v_code.ptr, t.code.data(), nnz * sizeof(int), cudaMemcpyHostToDevice, c.stream));
    }
    FORGE_CUDA(cudaMemcpyAsync(x->v_ph.ptr, ph.data(), ph.size() * sizeof(double2), cudaMemcpyHostToDevice, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    x->valley = true;
    return 0;
}

int forge_gpu_set_symmetry(forge_ctx* x, int64_t nenforceT, int64_t nenforceC2, int64_t nenforceC2T,
                           const int64_t* nC2pairs) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    auto flag = [](int64_t v) { return v == 0 || v == 1; };
    if (!flag(nenforceT) || !flag(nenforceC2) || !flag(nenforceC2T)) {
        set_error(FORGE_ERR_ARG, "set_symmetry: the switches are 0 or 1");
        return FORGE_ERR_ARG;
    }
    if (nenforceC2 || nenforceC2T) {
        // nC2pairs (C2_RelatedPoints, Geometry.f90:1140-1167) must pair every site
        const int64_t N = c.N;
        if (!nC2pairs) {
            set_error(FORGE_ERR_ARG, "set_symmetry: C2 / C2T need nC2pairs");
            return FORGE_ERR_ARG;
        }
        std::vector<char> seen(N, 0);
        std::vector<int64_t> perm(N);
        for (int64_t i = 0; i < N; ++i) {
            const int64_t j = nC2pairs[i];
            if (j < 1 || j > N || seen[j - 1]) {
                set_error(FORGE_ERR_ARG, "set_symmetry: nC2pairs is not a permutation of 1..%lld (site %lld)",
                          (long long)N, (long long)(i + 1));
                return FORGE_ERR_ARG;
            }
            seen[j - 1] = 1;
            perm[i] = j - 1;
        }
        FORGE_TRY(x->c2_perm.ensure(N * sizeof(int64_t)));
        FORGE_CUDA(cudaMemcpyAsync(x->c2_perm.ptr, perm.data(), N * sizeof(int64_t), cudaMemcpyHostToDevice,
                                   c.stream));
        FORGE_CUDA(cudaStreamSynchronize(c.stream));
    }
    x->sym_T = nenforceT == 1;
    x->sym_C2 = nenforceC2 == 1;
    x->sym_C2T = nenforceC2T == 1;
    return 0;
}

int forge_gpu_symmetrize(forge_ctx* x, double* zFock) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    FORGE_TRY(symmetrize_pnew(x));
    if (zFock)
        FORGE_CUDA(cudaMemcpyAsync(zFock, x->Pn.ptr, 4 * (size_t)c.N * c.N * sizeof(double2), cudaMemcpyDeviceToHost,
                                   c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

int forge_gpu_order_parameters(forge_ctx* x, const int64_t* nC2pairs, const int64_t* nC3pairs, double* out) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!out) {
        set_error(FORGE_ERR_ARG, "order_parameters: null output");
        return FORGE_ERR_ARG;
    }
    const int64_t N = c.N;
    // 0-based site maps; a map with a site left unpaired (0, as C2/C3_RelatedPoints leave it) is
    // not used and its norm is NaN
    std::vector<int64_t> maps(2 * N);
    bool ok[2] = {nC2pairs != nullptr, nC3pairs != nullptr};
    for (int t = 0; t < 2; ++t) {
        const int64_t* src = t == 0 ? nC2pairs : nC3pairs;
        for (int64_t i = 0; ok[t] && i < N; ++i) {
            if (src[i] < 1 || src[i] > N) ok[t] = false;
            else maps[t * N + i] = src[i] - 1;
        }
    }
    const int nblocks = 2 * 152;
    DevBuf dm, dpart;
    FORGE_TRY(dm.ensure(2 * N * sizeof(int64_t)));
    FORGE_TRY(dpart.ensure(nblocks * 4 * sizeof(double)));
    FORGE_CUDA(cudaMemcpyAsync(dm.ptr, maps.data(), 2 * N * sizeof(int64_t), cudaMemcpyHostToDevice, c.stream));
    const int64_t* m = dm.as<int64_t>();
    int rc = launch_order_params(c.stream, c.P.as<double2>(), N, c.s.nlayers, ok[0] ? m : nullptr,
                                 ok[1] ? m + N : nullptr, dpart.as<double>(), nblocks);
    std::vector<double> part(nblocks * 4);
    if (rc == 0) {
        cudaError_t e = cudaMemcpyAsync(part.data(), dpart.ptr, part.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                        c.stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
        if (e != cudaSuccess) {
            set_error(FORGE_ERR_CUDA, "order_parameters: %s", cudaGetErrorString(e));
            rc = FORGE_ERR_CUDA;
        }
    }
    dm.release();
    dpart.release();
    if (rc) return rc;
    double s[4] = {0, 0, 0, 0};
    for (int b = 0; b < nblocks; ++b)
        for (int t = 0; t < 4; ++t) s[t] += part[b * 4 + t];
    out[0] = s[0];
    out[1] = s[1];
    out[2] = ok[0] ? std::sqrt(s[2]) : NAN;
    out[3] = ok[1] ? std::sqrt(s[3]) : NAN;
    return 0;
}

int forge_gpu_set_mixing(forge_ctx* x, int64_t mode, int64_t depth, double beta) {
    FORGE_TRY(check_ctx(x));
    if ((mode != FORGE_MIX_ODA && mode != FORGE_MIX_PULAY && mode != FORGE_MIX_LINEAR) || depth < 1 ||
        depth > DIIS_MAX - 1 || !(beta > 0.0) ||
        beta > 1.0) {
        set_error(FORGE_ERR_ARG, "set_mixing: mode %lld, depth %lld (1..%d), beta %g (0..1]", (long long)mode,
                  (long long)depth, DIIS_MAX - 1, beta);
        return FORGE_ERR_ARG;
    }
    x->mix_mode = (int)mode;
    if (x->diis_depth != (int)depth) {
        x->diis_depth = (int)depth;
        x->diis_nslots = 0;
        x->diis_hist.release();
    }
    x->diis_beta = beta;
    diis_reset(x);
    return 0;
}

int forge_gpu_get_setup(forge_ctx* x, forge_setup* s) {
    FORGE_TRY(check_ctx(x));
    if (!s) {
        set_error(FORGE_ERR_ARG, "forge_gpu_get_setup: null setup");
        return FORGE_ERR_ARG;
    }
    *s = x->c.s;
    s->precision = x->c.precision;
    return 0;
}

int forge_gpu_timer_mark(forge_ctx* x, int64_t slot) {
    FORGE_TRY(check_ctx(x));
    if (slot < 0 || slot >= 64) {
        set_error(FORGE_ERR_ARG, "timer slot %lld out of range", (long long)slot);
        return FORGE_ERR_ARG;
    }
    if (!x->marks[slot]) FORGE_CUDA(cudaEventCreate(&x->marks[slot]));
    FORGE_CUDA(cudaEventRecord(x->marks[slot], x->c.stream));
    return 0;
}

int forge_gpu_timer_elapsed(forge_ctx* x, int64_t a, int64_t b, double* ms) {
    FORGE_TRY(check_ctx(x));
    if (a < 0 || a >= 64 || b < 0 || b >= 64 || !x->marks[a] || !x->marks[b] || !ms) {
        set_error(FORGE_ERR_ARG, "timer slots not recorded");
        return FORGE_ERR_ARG;
    }
    FORGE_CUDA(cudaEventSynchronize(x->marks[b]));
    float t = 0.f;
    FORGE_CUDA(cudaEventElapsedTime(&t, x->marks[a], x->marks[b]));
    *ms = t;
    return 0;
}

int forge_gpu_profile(forge_ctx* x, int64_t enable) {
    FORGE_TRY(check_ctx(x));
    x->prof.reset();
    x->prof.enabled = enable != 0;
    return 0;
}

int forge_gpu_profile_read(forge_ctx* x, double* ms, int64_t* launches, double* bytes, double* flops, int64_t n) {
    FORGE_TRY(check_ctx(x));
    x->prof.collect();
    const int64_t m = n < ST_COUNT ? n : ST_COUNT;
    for (int64_t s = 0; s < m; ++s) {
        if (ms) ms[s] = x->prof.ms[s];
        if (launches) launches[s] = x->prof.launches[s];
        if (bytes) bytes[s] = x->prof.bytes[s];
        if (flops) flops[s] = x->prof.flops[s];
    }
    return (int)ST_COUNT;
}

int forge_gpu_synchronize(forge_ctx* x) {
    FORGE_TRY(check_ctx(x));
    FORGE_CUDA(cudaStreamSynchronize(x->c.stream));
    return 0;
}

int forge_gpu_long_range(forge_ctx* x, double* LongRange) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    FORGE_TRY(launch_long_range(c));
    if (LongRange)
        FORGE_CUDA(cudaMemcpyAsync(LongRange, c.LR.ptr, (size_t)c.N * c.N * sizeof(double), cudaMemcpyDeviceToHost,
                                   c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

int forge_gpu_set_state(forge_ctx* x, const double* zFock) {
    FORGE_TRY(check_ctx(x));
    diis_reset(x);
    x->last_residual = INFINITY;
    x->oa_latched = false;
    if (!zFock) {
        set_error(FORGE_ERR_ARG, "forge_gpu_set_state: null zFock");
        return FORGE_ERR_ARG;
    }
    FORGE_TRY(upload_state(x, nullptr, zFock));
    FORGE_CUDA(cudaStreamSynchronize(x->c.stream));
    return 0;
}

int forge_gpu_get_state(forge_ctx* x, double* zFock, double* Density, double* Potential) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    const size_t NN = (size_t)c.N * c.N;
    if (zFock)
        FORGE_CUDA(cudaMemcpyAsync(zFock, c.P.ptr, 4 * NN * sizeof(double2), cudaMemcpyDeviceToHost, c.stream));
    if (Density) {
        FORGE_TRY(scf_density(c, c.P.as<double2>(), x->dens_new.as<double>()));
        FORGE_CUDA(cudaMemcpyAsync(Density, x->dens_new.ptr, c.N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    }
    if (Potential)
        FORGE_CUDA(cudaMemcpyAsync(Potential, c.V.ptr, c.N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

int forge_gpu_hamiltonian(forge_ctx* x, const double* Potential, const double* zFock, int64_t k0, int64_t nk,
                          double* H) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (k0 < 0 || nk < 1 || k0 + nk > c.Nk || !H) {
        set_error(FORGE_ERR_ARG, "forge_gpu_hamiltonian: bad k range");
        return FORGE_ERR_ARG;
    }
    FORGE_TRY(upload_state(x, Potential, zFock));
    const size_t NN = (size_t)c.N * c.N;
    DevBuf tmp;
    FORGE_TRY(tmp.ensure(nk * NN * sizeof(double2)));
    int rc = 0;
    if (cudaMemsetAsync(tmp.ptr, 0, nk * NN * sizeof(double2), c.stream) != cudaSuccess) rc = FORGE_ERR_CUDA;
    if (!rc) rc = launch_assemble(c, c.V.as<double>(), c.P.as<double2>(), k0, nk, tmp.as<double2>());
    if (!rc && cudaMemcpyAsync(H, tmp.ptr, nk * NN * sizeof(double2), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess)
        rc = FORGE_ERR_CUDA;
    if (!rc && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = FORGE_ERR_CUDA;
    if (rc == FORGE_ERR_CUDA) set_error(rc, "forge_gpu_hamiltonian: %s", cudaGetErrorString(cudaGetLastError()));
    tmp.release();
    return rc;
}

int forge_gpu_zheevr_batch(forge_ctx* x, int64_t nb, const double* A, int64_t iu, double* w, double* Z) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    const int64_t N = c.N;
    if (nb < 1 || iu < 1 || iu > N || !A || !w) {
        set_error(FORGE_ERR_ARG, "forge_gpu_zheevr_batch: bad arguments");
        return FORGE_ERR_ARG;
    }
    const size_t NN = (size_t)N * N;
    const bool oa = c.precision == FORGE_PREC_MIXED && x->oa_mode != 0;
    const int64_t iu_solve = oa ? N : iu;
    DevBuf dA, dX, dw, ws, mws, wall, ows, oerr;
    int rc = 0;
    if ((rc = dA.ensure(nb * NN * sizeof(double2))) || (rc = dX.ensure(nb * N * iu * sizeof(double2))) ||
        (rc = dw.ensure(nb * iu * sizeof(double))) || (rc = ws.ensure(eig_workspace_bytes(N, iu_solve, nb))))
        return rc;
    if (c.precision == FORGE_PREC_MIXED && (rc = mws.ensure(eig_mixed_workspace_bytes(N, iu_solve, nb)))) return rc;
    if (oa && ((rc = wall.ensure(nb * N * sizeof(double))) || (rc = ows.ensure(oa_workspace_bytes(N, iu))) ||
               (rc = oerr.ensure(sizeof(int)))))
        return rc;
    FORGE_CUDA(cudaMemcpyAsync(dA.ptr, A, nb * NN * sizeof(double2), cudaMemcpyHostToDevice, c.stream));
    EigArgs g{};
    g.n = N;
    g.iu = iu;
    g.batch = nb;
    g.A = dA.as<double2>();
    g.lda = N;
    g.strideA = N * N;
    g.X = dX.as<double2>();
    g.ldx = N;
    g.strideX = N * iu;
    g.w = dw.as<double>();
    g.ortol_rel = 1e-7;
    if (oa) {
        g.iu = N;
        g.iu_out = iu;
        g.w = wall.as<double>();
    }
    eig_bind_workspace(g, ws.ptr);
    rc = (c.precision == FORGE_PREC_MIXED) ? eig_mixed(c.stream, g, mws.ptr) : eig_fp64(c.stream, g);
    if (!rc && oa) {
        int64_t n4 = 0;
        const float* planes = eig_mixed_planes(mws.ptr, N, N, nb, &n4);
        cudaMemsetAsync(oerr.ptr, 0, sizeof(int), c.stream);
        rc = oa_refine(c.stream, g.A, g.strideA, planes, n4, N, g.w, N, iu, nb, g.X, g.ldx, g.strideX, dw.as<double>(),
                       iu, ows.ptr, oerr.as<int>(), x->oa_delta, x->oa_depth);
        int herr = 0;
        if (!rc && (cudaMemcpyAsync(&herr, oerr.ptr, sizeof(int), cudaMemcpyDeviceToHost, c.stream) != cudaSuccess ||
                    cudaStreamSynchronize(c.stream) != cudaSuccess || herr)) {
            set_error(FORGE_ERR_TIMEOUT, "eigenpair refinement: tensor-core wait gave up or CUDA error");
            rc = FORGE_ERR_TIMEOUT;
        }
        g.w = dw.as<double>();
        g.iu = iu;
    }
    DevBuf rws;
    if (!rc && c.precision == FORGE_PREC_MIXED && x->rr_width > 0) {
        // the same FP64 window refinement as the SCF's solves
        const int64_t nw = std::min<int64_t>(x->rr_width, iu);
        rc = rws.ensure(rr_window_workspace_bytes(N, nb));
        if (!rc)
            rc = rr_window(c.stream, g.A, g.strideA, g.X, g.ldx, g.strideX, g.w, iu, N, iu - nw, nw, nb, rws.ptr);
    }
    std::vector<int> fails(nb);
    if (!rc) {
        FORGE_CUDA(cudaMemcpyAsync(w, dw.ptr, nb * iu * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        if (Z) FORGE_CUDA(cudaMemcpyAsync(Z, dX.ptr, nb * N * iu * sizeof(double2), cudaMemcpyDeviceToHost, c.stream));
        FORGE_CUDA(cudaMemcpyAsync(fails.data(), g.fail, nb * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        FORGE_CUDA(cudaStreamSynchronize(c.stream));
    }
    dA.release();
    dX.release();
    dw.release();
    ws.release();
    mws.release();
    wall.release();
    ows.release();
    oerr.release();
    if (rc) return rc;
    int bad = 0;
    for (int64_t b = 0; b < nb; ++b) bad += fails[b] ? 1 : 0;
    return bad;
}

int forge_gpu_solve(forge_ctx* x, const double* Potential, const double* zFock, double* Bands, double* zEigenvectors,
                    double* zFockBulk) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    FORGE_TRY(upload_state(x, Potential, zFock));
    int info = 0;
    FORGE_TRY(solve_device(x, &info));
    const int64_t N = c.N, iu = c.nUpper, Nk = c.Nk, numb = c.numb;
    if (Bands) {
        std::vector<double> w((size_t)Nk * iu);
        FORGE_CUDA(cudaMemcpyAsync(w.data(), x->w.ptr, w.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        FORGE_CUDA(cudaStreamSynchronize(c.stream));
        for (int64_t k = 0; k < Nk; ++k)
            for (int64_t b = 0; b < numb; ++b) Bands[b + k * numb] = w[k * iu + c.nLower - 1 + b];
    }
    if (zEigenvectors) {
        for (int64_t k = 0; k < Nk; ++k)
            FORGE_CUDA(cudaMemcpyAsync(zEigenvectors + 2 * (size_t)k * N * numb,
                                       c.X.as<double2>() + (size_t)k * N * iu + (size_t)(c.nLower - 1) * N,
                                       (size_t)N * numb * sizeof(double2), cudaMemcpyDeviceToHost, c.stream));
    }
    if (zFockBulk)
        FORGE_CUDA(cudaMemcpyAsync(zFockBulk, c.bulk.ptr, 4 * (size_t)N * N * sizeof(double2), cudaMemcpyDeviceToHost,
                                   c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return info;
}

int forge_gpu_set_kshard(forge_ctx* x, int64_t k_begin, int64_t k_end) {
    FORGE_TRY(check_ctx(x));
    if (k_begin < 0 || k_end > x->c.Nk || k_begin >= k_end) {
        set_error(FORGE_ERR_ARG, "set_kshard: bad range [%lld, %lld)", (long long)k_begin, (long long)k_end);
        return FORGE_ERR_ARG;
    }
    x->k_begin = k_begin;
    x->k_end = k_end;
    return 0;
}

int forge_gpu_set_bands(forge_ctx* x, const double* Bands) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!x->have_solve || !Bands) {
        set_error(FORGE_ERR_STATE, "set_bands needs a solve first");
        return FORGE_ERR_STATE;
    }
    const int64_t iu = c.nUpper, numb = c.numb;
    for (int64_t k = 0; k < c.Nk; ++k)
        FORGE_CUDA(cudaMemcpyAsync(x->w.as<double>() + k * iu + c.nLower - 1, Bands + k * numb,
                                   numb * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    x->have_sort = false;
    return 0;
}

int forge_gpu_project_local(forge_ctx* x, double* zFock) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!x->have_sort) {
        set_error(FORGE_ERR_STATE, "project_local needs sort_energies / fermi first");
        return FORGE_ERR_STATE;
    }
    FORGE_TRY(project_fused(x));
    if (zFock)
        FORGE_CUDA(cudaMemcpyAsync(zFock, x->Pn.ptr, 4 * (size_t)c.N * c.N * sizeof(double2), cudaMemcpyDeviceToHost,
                                   c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

int forge_gpu_set_pnew(forge_ctx* x, const double* zFock) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!zFock) {
        set_error(FORGE_ERR_ARG, "set_pnew: null zFock");
        return FORGE_ERR_ARG;
    }
    const size_t NN = (size_t)c.N * c.N;
    FORGE_TRY(x->Pn.ensure(4 * NN * sizeof(double2)));
    FORGE_CUDA(cudaMemcpyAsync(x->Pn.ptr, zFock, 4 * NN * sizeof(double2), cudaMemcpyHostToDevice, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    x->have_pnew = true;
    return 0;
}

int forge_gpu_get_bands(forge_ctx* x, double* Bands) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!x->have_solve || !Bands) {
        set_error(FORGE_ERR_STATE, "get_bands needs a solve first");
        return FORGE_ERR_STATE;
    }
    const int64_t iu = c.nUpper, Nk = c.Nk, numb = c.numb;
    std::vector<double> w((size_t)Nk * iu);
    FORGE_CUDA(cudaMemcpyAsync(w.data(), x->w.ptr, w.size() * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    for (int64_t k = 0; k < Nk; ++k)
        for (int64_t b = 0; b < numb; ++b) Bands[b + k * numb] = w[k * iu + c.nLower - 1 + b];
    return 0;
}

int forge_gpu_sort_energies(forge_ctx* x, double* SortedEnergies, int64_t* nSortedMomenta, int64_t* nSortedIndex) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    FORGE_TRY(sort_device(x, c.s.nfilling));
    const int64_t nw = c.numb * c.Nk;
    std::vector<int64_t> idx(nw);
    FORGE_CUDA(cudaMemcpyAsync(idx.data(), x->sorted_idx.ptr, nw * sizeof(int64_t), cudaMemcpyDeviceToHost, c.stream));
    if (SortedEnergies)
        FORGE_CUDA(cudaMemcpyAsync(SortedEnergies, x->sorted_e.ptr, nw * sizeof(double), cudaMemcpyDeviceToHost,
                                   c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    x->h_sorted_idx = idx;
    if (nSortedIndex) std::memcpy(nSortedIndex, idx.data(), nw * sizeof(int64_t));
    if (nSortedMomenta) {
        for (int64_t q = 0; q < nw; ++q) {
            const int64_t icount = idx[q];
            const int64_t band = (icount - 1) / c.Nk, k = icount - 1 - band * c.Nk;
            nSortedMomenta[q] = c.kcomp[k];
            nSortedMomenta[q + nw] = c.kcomp[k + c.Nk];
        }
    }
    return 0;
}

int forge_gpu_fermi(forge_ctx* x, double nfilling, int64_t* nFermiLevel, double* FermiEnergy, int64_t* nOccStates,
                    int64_t* nPartOccStates, double* DegFactor) {
    FORGE_TRY(check_ctx(x));
    FORGE_TRY(sort_device(x, nfilling));
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    if (nFermiLevel) *nFermiLevel = h.nF;
    if (FermiEnergy) *FermiEnergy = h.EF;
    if (nOccStates) *nOccStates = h.nOcc;
    if (nPartOccStates) *nPartOccStates = h.nPart;
    if (DegFactor) *DegFactor = h.DegFactor;
    return 0;
}

int forge_gpu_get_fock(forge_ctx* x, double DegFactor, int64_t nOccStates, int64_t nPartOccStates, double* zFock) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!x->have_sort) {
        set_error(FORGE_ERR_STATE, "get_fock before sort_energies");
        return FORGE_ERR_STATE;
    }
    const int64_t nw = c.numb * c.Nk;
    if (nOccStates < 0 || nOccStates > nw || nPartOccStates < 0 || nPartOccStates > nOccStates) {
        set_error(FORGE_ERR_ARG, "get_fock: nOcc=%lld nPart=%lld out of range", (long long)nOccStates,
                  (long long)nPartOccStates);
        return FORGE_ERR_ARG;
    }
    // occupied window states with the caller's weights (HartreeFock.f90:506-555)
    std::vector<int64_t> idx(nw);
    FORGE_CUDA(cudaMemcpyAsync(idx.data(), x->sorted_idx.ptr, nw * sizeof(int64_t), cudaMemcpyDeviceToHost, c.stream));
    std::vector<double2> bph(c.Nk * 4);
    FORGE_CUDA(cudaMemcpyAsync(bph.data(), c.bphase.ptr, c.Nk * 4 * sizeof(double2), cudaMemcpyDeviceToHost, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    double2 zdeg = (c.s.degfactor_mode == FORGE_DEG_REFERENCE) ? make_double2((double)(float)DegFactor, 8.0)
                                                                : make_double2(DegFactor, 0.0);
    std::vector<WinState> st(nOccStates > 0 ? nOccStates : 1);
    for (int64_t q = 0; q < nOccStates; ++q) {
        const int64_t icount = idx[q];
        const int64_t band = (icount - 1) / c.Nk, k = icount - 1 - band * c.Nk;
        st[q].k = k;
        st[q].col = c.nLower - 1 + band;
        const double2 wgt = (q < nOccStates - nPartOccStates) ? make_double2(1.0, 0.0) : zdeg;
        for (int t = 0; t < 4; ++t) st[q].wph[t] = cmul(bph[k * 4 + t], wgt);
    }
    if (nOccStates == 0) st.clear();
    if (x->valley) {
        // Main.f90:470-511: the averaged window plus zFockBulk, divided by Nk
        const size_t NN = (size_t)c.N * c.N;
        FORGE_TRY(ensure_bulk(x));
        FORGE_TRY(x->Pn.ensure(4 * NN * sizeof(double2)));
        FORGE_CUDA(cudaMemsetAsync(x->Pn.ptr, 0, 4 * NN * sizeof(double2), c.stream));
        FORGE_TRY(valley_window(x, st));
        FORGE_TRY(scf_combine(c, x->Pn.as<double2>(), c.bulk.as<double2>()));
        x->have_pnew = true;
        if (zFock)
            FORGE_CUDA(cudaMemcpyAsync(zFock, x->Pn.ptr, 4 * NN * sizeof(double2), cudaMemcpyDeviceToHost, c.stream));
        FORGE_CUDA(cudaStreamSynchronize(c.stream));
        return 0;
    }
    expand_c3_states(x, st);
    const int64_t nst = (int64_t)st.size();
    if (nst > 0) {
        FORGE_TRY(x->states.ensure(nst * sizeof(WinState)));
        FORGE_CUDA(cudaMemcpyAsync(x->states.ptr, st.data(), nst * sizeof(WinState), cudaMemcpyHostToDevice,
                                   c.stream));
    }
    FORGE_TRY(get_fock_device(x, nst));
    if (zFock)
        FORGE_CUDA(cudaMemcpyAsync(zFock, x->Pn.ptr, 4 * (size_t)c.N * c.N * sizeof(double2), cudaMemcpyDeviceToHost,
                                   c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

int forge_gpu_energies(forge_ctx* x, const double* zFock, double* KineticEnergy, double* FockEnergy,
                       double* HartreeEnergy, double* HubbardEnergy) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!c.lr_ready) FORGE_TRY(launch_long_range(c));
    const size_t NN = (size_t)c.N * c.N;
    const double2* P = c.P.as<double2>();
    if (zFock) {
        FORGE_TRY(x->win.ensure(4 * NN * sizeof(double2)));
        FORGE_CUDA(cudaMemcpyAsync(x->win.ptr, zFock, 4 * NN * sizeof(double2), cudaMemcpyHostToDevice, c.stream));
        P = x->win.as<double2>();
    }
    double* d = x->dens_new.as<double>();
    FORGE_TRY(scf_density(c, P, d));
    ScfScalars keep;
    FORGE_TRY(read_scalars(x, &keep));
    FORGE_TRY(scf_energy_forms(c, x->te.as<double>(), P, P, d, d, x->y.as<double>(), x->work.as<double>(),
                               x->sc.as<ScfScalars>()));
    FORGE_TRY(scf_oda(c, x->sc.as<ScfScalars>(), 1));
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    if (KineticEnergy) *KineticEnergy = h.Eout[0];
    if (FockEnergy) *FockEnergy = h.Eout[1];
    if (HartreeEnergy) *HartreeEnergy = h.Eout[2];
    if (HubbardEnergy) *HubbardEnergy = h.Eout[3];
    FORGE_TRY(write_scalars(x, &keep));
    return 0;
}

int forge_gpu_optimal_step(forge_ctx* x, double* Step, double* Energies) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!x->have_pnew || !Energies) {
        set_error(FORGE_ERR_STATE, "optimal_step needs get_fock first and an Energies array");
        return FORGE_ERR_STATE;
    }
    if (!c.lr_ready) FORGE_TRY(launch_long_range(c));
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    for (int t = 0; t < 4; ++t) h.Ein[t] = Energies[t];
    FORGE_TRY(write_scalars(x, &h));
    FORGE_TRY(scf_density(c, x->Pn.as<double2>(), x->dens_new.as<double>()));
    FORGE_TRY(scf_energy_forms(c, x->te.as<double>(), c.P.as<double2>(), x->Pn.as<double2>(), c.dens.as<double>(),
                               x->dens_new.as<double>(), x->y.as<double>(), x->work.as<double>(),
                               x->sc.as<ScfScalars>()));
    FORGE_TRY(scf_oda(c, x->sc.as<ScfScalars>(), x->mix_mode == FORGE_MIX_LINEAR ? 2 : 0, x->diis_beta));
    FORGE_TRY(read_scalars(x, &h));
    if (Step) *Step = h.step;
    for (int t = 0; t < 4; ++t) Energies[t] = h.Eout[t];
    return 0;
}

int forge_gpu_energy_forms(forge_ctx* x, double* forms, double* Density, double* DensityNew) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!x->have_pnew || !forms) {
        set_error(FORGE_ERR_STATE, "energy_forms needs get_fock first and a forms array");
        return FORGE_ERR_STATE;
    }
    if (!c.lr_ready) FORGE_TRY(launch_long_range(c));
    // the density of the current state (the mix measures the density change against it)
    FORGE_TRY(scf_density(c, c.P.as<double2>(), c.dens.as<double>()));
    FORGE_TRY(scf_density(c, x->Pn.as<double2>(), x->dens_new.as<double>()));
    FORGE_TRY(scf_energy_forms(c, x->te.as<double>(), c.P.as<double2>(), x->Pn.as<double2>(), c.dens.as<double>(),
                               x->dens_new.as<double>(), x->y.as<double>(), x->work.as<double>(),
                               x->sc.as<ScfScalars>()));
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    for (int t = 0; t < 6; ++t) forms[t] = h.forms[t];
    if (Density)
        FORGE_CUDA(cudaMemcpyAsync(Density, c.dens.ptr, c.N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    if (DensityNew)
        FORGE_CUDA(
            cudaMemcpyAsync(DensityNew, x->dens_new.ptr, c.N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

int forge_gpu_mix_potential(forge_ctx* x, double Step, double* DensityConvergence, double* residual) {
    FORGE_TRY(check_ctx(x));
    Context& c = x->c;
    if (!x->have_pnew) {
        set_error(FORGE_ERR_STATE, "mix_potential needs get_fock / optimal_step first");
        return FORGE_ERR_STATE;
    }
    ScfScalars h;
    if (x->mix_mode == FORGE_MIX_PULAY) {
        // the Anderson / Pulay state replaces the OptimalStep mix (Step is not used); the energy
        // forms of (P_in, P_new) come from forge_gpu_optimal_step
        FORGE_TRY(pulay_mix(x));
    } else {
        FORGE_TRY(read_scalars(x, &h));
        h.step = Step;
        FORGE_TRY(write_scalars(x, &h));
        FORGE_TRY(scf_mix(c, c.P.as<double2>(), x->Pn.as<double2>(), c.dens.as<double>(), c.V.as<double>(),
                          x->y.as<double>(), x->work.as<double>(), x->sc.as<ScfScalars>()));
    }
    FORGE_TRY(read_scalars(x, &h));
    if (DensityConvergence) *DensityConvergence = h.dn_max;
    if (residual) *residual = h.residual;
    x->last_residual = h.residual;
    x->have_pnew = false;
    return 0;
}

int forge_gpu_plain_guess(forge_ctx* x, double* Energies) {
    FORGE_TRY(check_ctx(x));
    diis_reset(x);
    x->last_residual = INFINITY;
    x->oa_latched = false;
    Context& c = x->c;
    if (!c.lr_ready) FORGE_TRY(launch_long_range(c));
    const size_t NN = (size_t)c.N * c.N;
    FORGE_CUDA(cudaMemsetAsync(c.P.ptr, 0, 4 * NN * sizeof(double2), c.stream));
    FORGE_CUDA(cudaMemsetAsync(c.V.ptr, 0, c.N * sizeof(double), c.stream));
    int info = 0;
    FORGE_TRY(solve_device(x, &info, false));
    // Main.f90:255: nFermiLevel without the numS factor (numS = 1 here)
    FORGE_TRY(sort_device(x, c.s.nfilling));
    FORGE_TRY(project_fused(x));
    FORGE_CUDA(cudaMemcpyAsync(c.P.ptr, x->Pn.ptr, 4 * NN * sizeof(double2), cudaMemcpyDeviceToDevice, c.stream));
    x->have_pnew = false;
    FORGE_TRY(prepare_state_device(x, Energies));
    return info;
}

int forge_gpu_field_guess(forge_ctx* x, const double* zFock, double* Energies, double* residuals) {
    FORGE_TRY(check_ctx(x));
    diis_reset(x);
    x->last_residual = INFINITY;
    x->oa_latched = false;
    Context& c = x->c;
    if (!zFock || !residuals) {
        set_error(FORGE_ERR_ARG, "field_guess: null argument");
        return FORGE_ERR_ARG;
    }
    if (!c.lr_ready) FORGE_TRY(launch_long_range(c));
    const int64_t N = c.N;
    const size_t NN = (size_t)N * N;
    // predicted field: P_pred and V_pred = 2 alphaH LR dn + U dn from its diagonal
    FORGE_TRY(upload_state(x, nullptr, zFock));
    FORGE_TRY(scf_density(c, c.P.as<double2>(), c.dens.as<double>()));
    FORGE_TRY(scf_energy_forms(c, x->te.as<double>(), c.P.as<double2>(), c.P.as<double2>(), c.dens.as<double>(),
                               c.dens.as<double>(), x->y.as<double>(), x->work.as<double>(), x->sc.as<ScfScalars>()));
    FORGE_TRY(scf_potential(c, x->y.as<double>(), c.dens.as<double>(), c.V.as<double>()));
    std::vector<double> Vpred(N), V1(N);
    FORGE_CUDA(cudaMemcpyAsync(Vpred.data(), c.V.ptr, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    // one diagonalisation in that field (the cost of the plain guess)
    int info = 0;
    FORGE_TRY(solve_device(x, &info, false));
    FORGE_TRY(sort_device(x, c.s.nfilling));
    FORGE_TRY(project_fused(x));  // P_1 in Pn; c.bulk is all zeros afterwards
    // residuals of the predicted field and of the zero field against the field of P_1
    FORGE_TRY(scf_density(c, x->Pn.as<double2>(), x->dens_new.as<double>()));
    FORGE_TRY(scf_energy_forms(c, x->te.as<double>(), c.P.as<double2>(), x->Pn.as<double2>(), c.dens.as<double>(),
                               x->dens_new.as<double>(), x->y.as<double>(), x->work.as<double>(),
                               x->sc.as<ScfScalars>()));
    ScfScalars h;
    FORGE_TRY(read_scalars(x, &h));
    const double fock_ws = h.forms[5];
    FORGE_TRY(scf_energy_forms(c, x->te.as<double>(), c.bulk.as<double2>(), x->Pn.as<double2>(), c.dens.as<double>(),
                               x->dens_new.as<double>(), x->y.as<double>(), x->work.as<double>(),
                               x->sc.as<ScfScalars>()));
    FORGE_TRY(read_scalars(x, &h));
    const double fock_zero = h.forms[5];
    // V of P_1 (y holds LR dn_b from the last forms pass)
    FORGE_TRY(scf_potential(c, x->y.as<double>() + N, x->dens_new.as<double>(), c.V.as<double>()));
    FORGE_CUDA(cudaMemcpyAsync(V1.data(), c.V.ptr, N * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    FORGE_CUDA(cudaStreamSynchronize(c.stream));
    double dv_ws = 0.0, dv_zero = 0.0;
    for (int64_t i = 0; i < N; ++i) {
        dv_ws = std::max(dv_ws, std::fabs(V1[i] - Vpred[i]));
        dv_zero = std::max(dv_zero, std::fabs(V1[i]));
    }
    residuals[0] = std::max(dv_ws, fock_ws);
    residuals[1] = std::max(dv_zero, fock_zero);
    // the state becomes P_1 (Main.f90:281-346 with the predicted field in place of zero)
    FORGE_CUDA(cudaMemcpyAsync(c.P.ptr, x->Pn.ptr, 4 * NN * sizeof(double2), cudaMemcpyDeviceToDevice, c.stream));
    x->have_pnew = false;
    FORGE_TRY(prepare_state_device(x, Energies));
    return info;
}

int forge_gpu_prepare_state(forge_ctx* x, double* Energies) {
    FORGE_TRY(check_ctx(x));
    diis_reset(x);
    x->last_residual = INFINITY;
    x->oa_latched = false;
    Context& c = x->c;
    if (!c.lr_ready) FORGE_TRY(launch_long_range(c));
    return prepare_state_device(x, Energies);
}

int forge_gpu_set_potential(forge_ctx* x, const double* Potential) {
    FORGE_TRY(check_ctx(x));
    if (!Potential) {
        set_error(FORGE_ERR_ARG, "set_potential: null Potential");
        return FORGE_ERR_ARG;
    }
    FORGE_TRY(upload_state(x, Potential, nullptr));
    FORGE_CUDA(cudaStreamSynchronize(x->c.stream));
    return 0;
}

int forge_gpu_solve_group(forge_ctx** ctxs, int64_t nctx, int64_t* info) {
    if (!ctxs || nctx < 1) {
        set_error(FORGE_ERR_ARG, "solve_group: no contexts");
        return FORGE_ERR_ARG;
    }
    for (int64_t b = 0; b < nctx; ++b) FORGE_TRY(check_ctx(ctxs[b]));
    FORGE_TRY(check_ctx(ctxs[0]));
    std::vector<int> infos(nctx, 0);
    FORGE_TRY(solve_group_device(ctxs, nctx, infos.data()));
    int bad = 0;
    for (int64_t b = 0; b < nctx; ++b) {
        if (info) info[b] = infos[b];
        bad += infos[b];
    }
    return bad;
}

int forge_gpu_scf_iteration_group(forge_ctx** ctxs, int64_t nctx, double* Energies, forge_iter_report* reports) {
    if (!ctxs || nctx < 1) {
        set_error(FORGE_ERR_ARG, "scf_iteration_group: no contexts");
        return FORGE_ERR_ARG;
    }
    std::vector<double> Ein(4 * nctx);
    for (int64_t b = 0; b < nctx; ++b) {
        FORGE_TRY(check_ctx(ctxs[b]));
        FORGE_TRY(scf_iteration_begin(ctxs[b], Energies ? Energies + 4 * b : nullptr, &Ein[4 * b]));
    }
    FORGE_TRY(check_ctx(ctxs[0]));
    std::vector<int> infos(nctx, 0);
    FORGE_TRY(solve_group_device(ctxs, nctx, infos.data()));
    int bad = 0;
    for (int64_t b = 0; b < nctx; ++b) {
        FORGE_TRY(check_ctx(ctxs[b]));
        FORGE_TRY(scf_iteration_end(ctxs[b], &Ein[4 * b], infos[b], Energies ? Energies + 4 * b : nullptr,
                                    reports ? reports + b : nullptr));
        bad += infos[b];
    }
    return bad;
}

int forge_gpu_scf_iteration(forge_ctx* x, double* Energies, forge_iter_report* rep) {
    FORGE_TRY(check_ctx(x));
    double Ein[4];
    FORGE_TRY(scf_iteration_begin(x, Energies, Ein));
    int info = 0;
    FORGE_TRY(solve_device(x, &info, false));
    FORGE_TRY(scf_iteration_end(x, Ein, info, Energies, rep));
    return info;
}

}  // extern "C"
