/*
 * forge_gpu.h -- C-ABI of the GB300 (sm_103a) Hartree-Fock SCF engine.
 *
 * Drop-in boundary for the hot path of FORGE (forge-team/forge, Fortran 90):
 * every entry point replaces one routine of HartreeFock.f90 / LapackRoutines.f90
 * or one inline loop of Main.f90, with the same argument meaning.  A Fortran
 * host binds these with ISO_C_BINDING.
 *
 * Conventions
 *   - integers are int64_t (the reference's integer(dp)), reals are double (real(dp));
 *   - complex arrays are interleaved (re, im) doubles, i.e. Fortran complex(dp) /
 *     C99 double _Complex, column-major, 1-based indices in the reference map to
 *     0-based offsets here;
 *   - zFock-shaped arrays are ndim x ndim x numNeighborCells (Main.f90:104-106);
 *   - a NULL host pointer for an input means "use the device-resident copy kept
 *     by the context"; a NULL host pointer for an output means "keep it on the
 *     device only" (no host copy);
 *   - every call returns a status: 0 = OK, > 0 = eigen-solver info (LAPACK style,
 *     number of k points whose solve did not converge), < 0 = FORGE_ERR_*.
 *     forge_gpu_last_error() gives the message of the last failure.
 *   - a context is used from one host thread at a time; all work runs on the
 *     context's own CUDA stream.
 */
#ifndef FORGE_GPU_H
#define FORGE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    FORGE_OK = 0,
    FORGE_ERR_ARG = -1,     /* invalid argument */
    FORGE_ERR_CUDA = -2,    /* CUDA runtime error */
    FORGE_ERR_STATE = -3,   /* call out of order (e.g. solve before init) */
    FORGE_ERR_NOMEM = -4,   /* device allocation failed */
    FORGE_ERR_TIMEOUT = -5, /* a bounded device-side wait gave up */
    FORGE_ERR_NUMERIC = -6  /* non-finite value detected */
};

enum { FORGE_PREC_FP64 = 0, FORGE_PREC_MIXED = 1 };
/* SCF mixing: the reference's OptimalStep (ODA) or Anderson / Pulay mixing of the density matrix. */
enum { FORGE_MIX_ODA = 0, FORGE_MIX_PULAY = 1, FORGE_MIX_LINEAR = 2 };
enum { FORGE_DEG_REFERENCE = 0, FORGE_DEG_CORRECTED = 1 };

/* Runtime mirror of Setup.f90:6-74 (only the parameters the SCF path reads). */
typedef struct forge_setup {
    int64_t nlayers;          /* Setup.f90:7 */
    int64_t ntheta;           /* Setup.f90:8 */
    int64_t numk;             /* Setup.f90:11 */
    int64_t numS;             /* Setup.f90:13: a context holds one spin (1); numS = 2 runs one context per
                                 spin joined on the host (forge_host_fermi_2spins) */
    int64_t numI;             /* Setup.f90:19 (only 1 is supported: 4 neighbour cells) */
    int64_t numC;             /* Setup.f90:20 */
    int64_t nscreen;          /* Setup.f90:21 */
    int64_t fphase;           /* Setup.f90:25 (only 0: the projectors apply no site phase) */
    int64_t ndim;             /* Setup.f90:10 */
    int64_t numb;             /* Setup.f90:23 */
    int64_t nLower, nUpper;   /* Setup.f90:67-68 */
    int64_t NeutralityPoint;  /* Setup.f90:69 */
    int64_t numNeighborCells; /* Geometry.f90:14-35 */
    int64_t degfactor_mode;   /* FORGE_DEG_*: zdeg of HartreeFock.f90:529 */
    int64_t precision;        /* FORGE_PREC_*: eigen-solver / projector arithmetic */
    double nfilling;          /* Setup.f90:14 */
    double U;                 /* Setup.f90:16 */
    double epsilon;           /* Setup.f90:17 */
    double Delta;             /* Setup.f90:18 */
    double xi;                /* Setup.f90:22 */
    double alpha, alphaH;     /* Setup.f90:58-59 */
    double a0, r0, d0, tz;    /* Setup.f90:62-65 */
    double EnergyTolerance;   /* Setup.f90:51 */
    double StepAlternative;   /* Setup.f90:52 */
} forge_setup;

typedef struct forge_ctx forge_ctx;

/* Per-iteration report of forge_gpu_scf_iteration (the Convergence / Energy
 * lines of Main.f90:616-639 plus the Fermi bookkeeping of Main.f90:400-412). */
typedef struct forge_iter_report {
    double Step;              /* ODA step (HartreeFock.f90:1201-1208) */
    double DensityConvergence;/* max |n - n_in| (Main.f90:564-571) */
    double TotalEnergyIn, TotalEnergy;
    double KineticEnergyIn, FockEnergyIn, HartreeEnergyIn, HubbardEnergyIn;
    double KineticEnergy, FockEnergy, HartreeEnergy, HubbardEnergy;
    double FermiEnergy, DegFactor;
    double residual;          /* max change of any H_HF element (eV) */
    int64_t nFermiLevel, nOccStates, nPartOccStates;
    int64_t info;             /* eigen-solver info of this iteration */
    int64_t refined;          /* 1 if this iteration's eigenpairs were refined (forge_gpu_set_eigen_refinement) */
} forge_iter_report;

const char* forge_gpu_last_error(void);
int forge_gpu_version(void);
/* Number of kernels this library has launched in the process so far (all contexts). */
int64_t forge_gpu_launch_count(void);

/* Creates a context: uploads the geometry built by the host (Main.f90:123-154) and
 * tabulates ft / fv for the 7 cell images (K1).  tn = [t1, t2, t3] as a 2x3 column-major
 * array (Main.f90:249 reshape([t1,t2,t3],[2,3])). */
int forge_gpu_init(const forge_setup* setup, const double* Coords, const int64_t* nUnitCell_1,
                   const int64_t* nUnitCell_2, const double* tn, const double* MomentaValues,
                   const int64_t* nMomentaComponents, forge_ctx** ctx);
int forge_gpu_finalize(forge_ctx* ctx);

/* LongRangeInteraction (HartreeFock.f90:14-53).  LongRange (ndim x ndim) may be NULL. */
int forge_gpu_long_range(forge_ctx* ctx, double* LongRange);

/* Loads zFock (and its density Re diag zFock(:,:,1)) as the current state P = zFockIn,
 * e.g. after reading a checkpoint (Main.f90:202-234) or a learned warm start. */
int forge_gpu_set_state(forge_ctx* ctx, const double* zFock);
/* Copies the current state back: zFock (ndim x ndim x NNC complex), Density (ndim),
 * Potential (ndim); any of them may be NULL. */
int forge_gpu_get_state(forge_ctx* ctx, double* zFock, double* Density, double* Potential);

/* HamiltonianHartreeFock (HartreeFock.f90:57-127) for k points [k0, k0+nk): writes the
 * lower triangles of H(k) (ndim x ndim complex each) to H (host).  Potential / zFock NULL =
 * device state. */
int forge_gpu_hamiltonian(forge_ctx* ctx, const double* Potential, const double* zFock, int64_t k0,
                          int64_t nk, double* H);

/* zdiagRed (LapackRoutines.f90:381-433) on a batch of nb Hermitian matrices given in the
 * lower triangle (ndim x ndim complex each, column-major, host): eigenvalues 1..iu in
 * ascending order into w (iu x nb) and eigenvectors into Z (ndim x iu x nb). */
int forge_gpu_zheevr_batch(forge_ctx* ctx, int64_t nb, const double* A, int64_t iu, double* w, double* Z);

/* Solve (HartreeFock.f90:402-483): H(k) for all k, eigenpairs 1..nUpper, window bands and
 * vectors, bulk projector zFockBulk (NOT divided by Nk, as in the reference). */
int forge_gpu_solve(forge_ctx* ctx, const double* Potential, const double* zFock, double* Bands,
                    double* zEigenvectors, double* zFockBulk);

/* Bands (numb x Nk) of the last Solve or SCF iteration (HartreeFock.f90:444-446). */
int forge_gpu_get_bands(forge_ctx* ctx, double* Bands);

/* k-point sharding across ranks (the reference's OpenMP k loop, HartreeFock.f90:424-478, split
 * over GPUs).  set_kshard restricts Solve and the projectors to flat k in [k_begin, k_end);
 * set_bands installs the all-gathered Bands (numb x Nk) before the sort so every rank finds the
 * same Fermi level; project_local forms this rank's share of P_new = (window + bulk)/Nk over its
 * k points (zFock: host copy, NULL allowed), and set_pnew loads the all-reduced P_new for
 * forge_gpu_optimal_step / forge_gpu_mix_potential. */
int forge_gpu_set_kshard(forge_ctx* ctx, int64_t k_begin, int64_t k_end);
int forge_gpu_set_bands(forge_ctx* ctx, const double* Bands);
int forge_gpu_project_local(forge_ctx* ctx, double* zFock);
int forge_gpu_set_pnew(forge_ctx* ctx, const double* zFock);

/* SortEnergies_1Spin (HartreeFock.f90:885-925) of the last Solve: SortedEnergies (numb*Nk),
 * nSortedMomenta (numb*Nk x 2), nSortedIndex (numb*Nk, the reference's flattened index
 * icount = (band-1)*Nk + k, 1-based); any output may be NULL. */
int forge_gpu_sort_energies(forge_ctx* ctx, double* SortedEnergies, int64_t* nSortedMomenta,
                            int64_t* nSortedIndex);

/* Fermi level and degeneracy bookkeeping (Main.f90:400-412) on the last sort. */
int forge_gpu_fermi(forge_ctx* ctx, double nfilling, int64_t* nFermiLevel, double* FermiEnergy,
                    int64_t* nOccStates, int64_t* nPartOccStates, double* DegFactor);

/* GetFock (HartreeFock.f90:487-560) followed by Main.f90:510-511: the new density matrix
 * P_new = (window projector + zFockBulk)/Nk, kept on the device; zFock (NULL allowed)
 * receives a host copy. */
int forge_gpu_get_fock(forge_ctx* ctx, double DegFactor, int64_t nOccStates, int64_t nPartOccStates,
                       double* zFock);

/* GetKineticEnergy + GetFockEnergy + GetHartreeHubbardEnergy (HartreeFock.f90:1012-1145) of
 * zFock (NULL = device state P) with Density-1/2 from Re diag zFock(:,:,1). */
int forge_gpu_energies(forge_ctx* ctx, const double* zFock, double* KineticEnergy, double* FockEnergy,
                       double* HartreeEnergy, double* HubbardEnergy);

/* OptimalStep (HartreeFock.f90:1148-1227) on the device pair (P_new, P_in); Energies[4] holds
 * (Kinetic, Fock, Hartree, Hubbard) of P_in on entry and of the stepped state on exit. */
int forge_gpu_optimal_step(forge_ctx* ctx, double* Step, double* Energies);

/* The energy forms of the current state P_in and of P_new (after forge_gpu_get_fock), from which the
 * kinetic and Fock energies of every mix (1-s) P_in + s P_new follow (OptimalStep's three
 * evaluations, HartreeFock.f90:1148-1227, of one spin of a numS = 2 run): forms[0] = E_kin(P_in),
 * forms[1] = E_kin(P_new), forms[2..4] = Q(P_in, P_in), Q(P_in, P_new), Q(P_new, P_new) with
 * E_Fock(P) = -Q(P, P) / 2, forms[5] = max alpha |fv| |P_new - P_in| (6 doubles).  Density and
 * DensityNew (N each, may be NULL) receive the site densities of P_in and P_new.  Nothing is mixed:
 * forge_gpu_mix_potential with the chosen step follows. */
int forge_gpu_energy_forms(forge_ctx* ctx, double* forms, double* Density, double* DensityNew);

/* Main.f90:558-595: P = Step*P_new + (1-Step)*P_in, Density, DensityConvergence, Potential;
 * P_in <- P.  residual receives the mean-field residual (NULL allowed).  With FORGE_MIX_PULAY
 * (forge_gpu_set_mixing) the new state is the Anderson / Pulay mix of the history instead and
 * Step is not used; forge_gpu_optimal_step must still come first (its energy-forms pass of
 * (P_in, P_new) feeds the Pulay residual), as in the reference's call order. */
int forge_gpu_mix_potential(forge_ctx* ctx, double Step, double* DensityConvergence, double* residual);

/* Initial guess without a checkpoint (Main.f90:236-346, nRead=0): non-interacting Solve,
 * sort, Fermi, GetFock, energies and potential.  Energies[4] as in optimal_step. */
int forge_gpu_plain_guess(forge_ctx* ctx, double* Energies);

/* Initial guess from a predicted mean field (no counterpart in the reference): zFock holds the
 * predicted density matrix (e.g. a learned warm start on short bonds plus site densities); its
 * field is diagonalised once like the plain guess, and the resulting density matrix becomes the
 * state.  residuals[0] = residual of the predicted field, residuals[1] = residual of the zero
 * field (the plain guess), both against the field of the new state; Energies[4] as in
 * forge_gpu_optimal_step. */
int forge_gpu_field_guess(forge_ctx* ctx, const double* zFock, double* Energies, double* residuals);

/* After forge_gpu_set_state: energies and potential of the loaded state (Main.f90:290-346). */
int forge_gpu_prepare_state(forge_ctx* ctx, double* Energies);

/* One full SCF iteration (Main.f90:365-595) with all arrays device-resident.
 * Energies[4] as in optimal_step (in: current, out: new). */
int forge_gpu_scf_iteration(forge_ctx* ctx, double* Energies, forge_iter_report* report);

/* Uneven-size batch (no counterpart in the reference, which builds one system per binary,
 * Setup.f90:6-74): the Solve eigen-step of nctx contexts of different ndim (same precision, same
 * device, no C3 / valley / k shard / eigenpair refinement) as ONE batched eigen-solve.  Every H(k)
 * of every context is embedded in an nmax x nmax slot (nmax = the largest ndim) with a Gershgorin
 * shift s > every eigenvalue on the padded diagonal, which decouples exactly, so each context gets
 * the eigenpairs 1..nUpper of its own H(k) (plus the FP64 window Rayleigh-Ritz of its own window in
 * mixed precision).  info[b] (NULL allowed): number of k of context b whose solve did not converge.
 * The work runs on ctxs[0]'s stream and its group buffers. */
int forge_gpu_solve_group(forge_ctx** ctxs, int64_t nctx, int64_t* info);
/* Loads Potential (ndim) as the potential of the next solve without solving (the Potential argument
 * of Solve, HartreeFock.f90:402-411, for hosts that batch several contexts' solves with
 * forge_gpu_solve_group, e.g. the two spins of numS = 2). */
int forge_gpu_set_potential(forge_ctx* ctx, const double* Potential);
/* One SCF iteration of each context (forge_gpu_scf_iteration) with the eigen-solve shared as in
 * forge_gpu_solve_group: Energies is nctx x 4 (NULL allowed), reports nctx (NULL allowed). */
int forge_gpu_scf_iteration_group(forge_ctx** ctxs, int64_t nctx, double* Energies, forge_iter_report* reports);

/* Mixing of forge_gpu_scf_iteration (no counterpart in the reference, which mixes with OptimalStep
 * only):
 * FORGE_MIX_ODA (default) or FORGE_MIX_PULAY with `depth` (1..7) previous steps and mixing weight
 * beta (0..1]: P_in <- P_in + beta r - sum_i g_i (dP_i + beta dr_i), r = P_new - P_in, with g
 * minimising |r - sum_i g_i dr_i|.  The history (complex64 differences, 2 x 4 N^2 x 8 bytes per
 * step) is kept on the device and is cleared by set_state, plain_guess, field_guess,
 * prepare_state and a change of precision.  With Pulay the reported residual is that of
 * (P_in, P_new) and Step is 1.  FORGE_MIX_LINEAR mixes P <- beta P_new + (1 - beta) P_in (the
 * benchmark description's "linear mixing 0.3"): forge_gpu_optimal_step then returns Step = beta
 * with the energies of that state, and depth is not used. */
int forge_gpu_set_mixing(forge_ctx* ctx, int64_t mode, int64_t depth, double beta);

/* FP64 Rayleigh-Ritz refinement after every FORGE_PREC_MIXED eigen-solve (no counterpart in the
 * reference): the top `width` computed eigenvectors of each k (the zdiagRed window and the bands
 * below it, width 0..32, default 32, 0 = off) are re-solved in their span with FP64 products
 * against the FP64 H(k): Y = H X, G = X^H Y, S = X^H X, then G z = theta S z on the host. */
int forge_gpu_set_refinement(forge_ctx* ctx, int64_t width);

/* Eigenpair refinement of the FORGE_PREC_MIXED eigen-solve (no counterpart in the reference, whose
 * zheevr is FP64 throughout, LapackRoutines.f90:414-426): the mixed solve computes all ndim
 * eigenpairs, then one Ogita-Aishima correction step makes eigenpairs 1..nUpper FP64-accurate.  The
 * residual H X - X lam is an error-free product of integer slices on the tensor cores; the
 * correction E = (X^H W) / (lam_j - lam_i) and X += X E use TF32 hi/lo products; pairs closer than
 * delta (eV, default 1e-3) are only orthogonalised (FP64 overlaps).  The FP64 window Rayleigh-Ritz
 * (forge_gpu_set_refinement) runs after it.  mode 0 = off (default), 1 = every mixed solve, 2 = the
 * SCF solves from the first one after a residual below residual_below (eV) until the next guess or
 * state load (forge_gpu_plain_guess, _field_guess, _set_state, _prepare_state).  depth 1..4 (0 = default 4):
 * slice products s + t <= depth, relative accuracy of the residual ~2^-(25 + 9 depth). */
int forge_gpu_set_eigen_refinement(forge_ctx* ctx, int64_t mode, double residual_below, double delta,
                                   int64_t depth);
/* 1 if the last solve's eigenpairs were refined (for hosts that call forge_gpu_solve directly). */
int forge_gpu_last_refined(forge_ctx* ctx, int64_t* refined);

/* nenforceC3 (Setup.f90:27): 1 selects Solve_C3 / GetFock_C3 (HartreeFock.f90:131-398, 564-881) in
 * every later solve and projector; 0 (the default) the full solve.  nC3pairs is the 1-based site map
 * of C3_RelatedPoints (Geometry.f90:1172-1223, a permutation), RotateLayers the nlayers layer
 * rotations (Setup.f90).  H(k) is solved only for the first k of each C3 orbit; the other two k get
 * the representative's eigenvectors with rows permuted by nC3pairs and the corner sites phased, and
 * at the three C3-invariant k the projectors are the average of the k's projector and its two
 * rotated copies.  Needs numk divisible by 3 and fphase = 0 (FORGE_ERR_ARG otherwise), and no k shard. */
int forge_gpu_set_c3(forge_ctx* ctx, int64_t nenforceC3, const int64_t* nC3pairs, const int64_t* RotateLayers);

/* nenforceValley (Setup.f90:31): 1 averages the window part of every new density matrix of the SCF
 * loop (forge_gpu_scf_iteration, forge_gpu_get_fock; not the initial guess) with its valley
 * transform, as Main.f90:470-500 does: GetFock over the window eigenvectors X and over X S(k),
 * S(k) = sign(X^H V(k) X) with the valley operator V(k) of ValleyPhase (TightBinding.f90:60-157),
 * each with weight 1/2.  RotateLayers (nlayers) gives each layer's rotation.  Not combined with the
 * C3-reduced solve or a k shard (FORGE_ERR_ARG / FORGE_ERR_STATE). */
int forge_gpu_set_valley(forge_ctx* ctx, int64_t nenforceValley, const int64_t* RotateLayers);

/* nenforceT, nenforceC2, nenforceC2T (Setup.f90:28-30), each 0 (default) or 1: the symmetry
 * averages of Main.f90:513-534 on every new density matrix of forge_gpu_scf_iteration (not on the
 * initial guess), in the order T, C2, C2T.  nC2pairs (1-based, a permutation; C2_RelatedPoints,
 * Geometry.f90:1140-1167) is read when C2 or C2T is on and may be NULL otherwise. */
int forge_gpu_set_symmetry(forge_ctx* ctx, int64_t nenforceT, int64_t nenforceC2, int64_t nenforceC2T,
                           const int64_t* nC2pairs);

/* The same averages on the device P_new of forge_gpu_get_fock, for hosts that call the routines one
 * by one; copies the result to zFock when it is not NULL. */
int forge_gpu_symmetrize(forge_ctx* ctx, double* zFock);

/* Order parameters of the current state P(R=0) (no counterpart in the reference, which computes
 * none; defined from P and the site maps of C2_RelatedPoints / C3_RelatedPoints,
 * Geometry.f90:1140-1223): out[0] layer polarisation sum_l (l - (L-1)/2) sum_{i in l} (n_i - 1/2),
 * out[1] sublattice polarisation (A block minus B block of every layer), out[2] the C2T breaking
 * norm ||P0(i,j) - P0(c2(j),c2(i))||_F, out[3] the C3 breaking norm ||P0(i,j) - P0(c3(i),c3(j))||_F.
 * nC2pairs / nC3pairs are 1-based; a map that is NULL or leaves a site unpaired gives NaN. */
int forge_gpu_order_parameters(forge_ctx* ctx, const int64_t* nC2pairs, const int64_t* nC3pairs, double* out);

/* Selects FORGE_PREC_FP64 or FORGE_PREC_MIXED for subsequent solves. */
int forge_gpu_set_precision(forge_ctx* ctx, int64_t precision);

/* Copies the context's setup (as passed to forge_gpu_init, with the current precision). */
int forge_gpu_get_setup(forge_ctx* ctx, forge_setup* setup);

/* Stage timing with CUDA events on the context's stream (no counterpart in the reference,
 * which has no timers).  forge_gpu_profile(ctx, 1) resets and enables it; profile_read fills
 * up to n entries per stage (milliseconds, launches, algorithmic bytes and flops) in the
 * order: tables, long_range, assemble, trd_col, hemv, trd_finish, her2k, bisect, invit,
 * backtransform, projector, window, sort, energy, lr_matvec, mix, refine; returns the
 * number of stages. */
int forge_gpu_profile(forge_ctx* ctx, int64_t enable);
/* Records a CUDA event in slot (0..63) on the context stream / elapsed ms between two slots. */
int forge_gpu_timer_mark(forge_ctx* ctx, int64_t slot);
int forge_gpu_timer_elapsed(forge_ctx* ctx, int64_t slot_a, int64_t slot_b, double* ms);
int forge_gpu_profile_read(forge_ctx* ctx, double* ms, int64_t* launches, double* bytes, double* flops,
                           int64_t n);

/* Learned SCF warm start (no counterpart in the reference, which starts from the non-interacting
 * guess or a checkpoint): an MLP din -> 128 -> 128 -> 128 -> dout (SiLU), BF16 weights, FP32
 * accumulation and master weights, trained with Adam by hand-written kernels.  X: n x din,
 * targets / outputs: n x dout, row-major fp32 host arrays.  Loss: sum_o wt_o (y_o - t_o)^2 / n. */
typedef struct forge_mlp forge_mlp;
int forge_gpu_mlp_create(int64_t din, int64_t dout, uint64_t seed, forge_mlp** mlp);
int forge_gpu_mlp_destroy(forge_mlp* mlp);
int64_t forge_gpu_mlp_num_params(forge_mlp* mlp);
int forge_gpu_mlp_set_params(forge_mlp* mlp, const float* params);
int forge_gpu_mlp_get_params(forge_mlp* mlp, float* params, float* params_bf16);
int forge_gpu_mlp_set_loss_weights(forge_mlp* mlp, const float* wt);
int forge_gpu_mlp_forward(forge_mlp* mlp, const float* X, int64_t n, float* Y);
int forge_gpu_mlp_gradient(forge_mlp* mlp, const float* X, const float* targets, int64_t n, float* grad,
                           float* loss);
int forge_gpu_mlp_train(forge_mlp* mlp, const float* X, const float* targets, int64_t n, int64_t epochs,
                        int64_t batch, double lr, uint64_t seed, float* last_loss);

/* Allocation-free eigen-solver (no counterpart in the reference): zdiagRed for one Hermitian
 * matrix (lower triangle of A, n x n complex, column-major) for callers that cannot allocate
 * device memory at call time (a memory pool or arena owning the whole GPU, hosts that manage
 * every device buffer themselves).  A (overwritten), w (iu eigenvalues) and Z (n x iu complex
 * eigenvectors) are DEVICE pointers; stream is a cudaStream_t (NULL = default stream).  The
 * workspace is a static device array of FORGE_NOALLOC_SCRATCH_BYTES held by every GPU that loads
 * the library, so 2 <= n <= FORGE_NOALLOC_MAX_N; other n are rejected with FORGE_ERR_ARG (n = 1
 * needs no solver: w = Re A, Z = 1).  The first call on a device looks up the array's device
 * address.  Every call ends by synchronising `stream` to read the solver's convergence flag, so
 * the call blocks the host until its work is done and cannot be recorded into a CUDA graph.
 * Calls share the array: calls whose work overlaps on the GPU race.  Returns 0, 1 (inverse
 * iteration did not converge) or FORGE_ERR_*.  The solver is the FP64 path of
 * forge_gpu_zheevr_batch. */
#define FORGE_NOALLOC_MAX_N 512
#define FORGE_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)
int forge_gpu_zheevr_noalloc(double* A, int64_t n, int64_t iu, double* w, double* Z, void* stream);

/* Synchronises the context's stream (for host timing). */
int forge_gpu_synchronize(forge_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* FORGE_GPU_H */
