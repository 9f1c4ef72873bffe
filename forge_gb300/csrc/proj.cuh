// Projector and SCF-scalar kernels shared between the plain and mixed paths.
#pragma once
#include "forge_internal.cuh"

namespace forge {

// One occupied window state of GetFock (HartreeFock.f90:506-555): its k point, the
// column of X_k holding its eigenvector, and weight * Bloch phase for the four cells.
struct WinState {
    int64_t k;
    int64_t col;
    double2 wph[4];
};

int bulk_projector_fp64(cudaStream_t st, const double2* X, int64_t ldx, int64_t N, int64_t K, const double2 ph[4],
                        double2* P);
int window_projector_fp64(cudaStream_t st, const WinState* states, int64_t nstates, const double2* X, int64_t ldx,
                          int64_t strideX, int64_t N, double2* P);
size_t proj_tc_workspace_floats(int64_t n, int64_t iu);
int bulk_projector_tc(cudaStream_t st, const double2* X, int64_t ldx, int64_t n, int64_t K, int64_t iu,
                      const double2 ph[4], double2* P, float* ws, int* err);
size_t proj_tc_exact_workspace_bytes(int64_t n, int64_t iu);
int bulk_projector_tc_exact(cudaStream_t st, const double2* X, int64_t ldx, int64_t n, int64_t K, int64_t iu,
                            const double2 ph[4], double2* P, void* ws, int* err);

// Device scalars of one SCF iteration (filled by k_sort_fermi / k_oda).
struct ScfScalars {
    double EF, DegFactor;
    int64_t nF, nOcc, nPart, nStates;
    double zdeg_re, zdeg_im;
    // energy forms: [0] Kin_a [1] Kin_b [2] Qaa [3] Qab [4] Qbb [5] Mres (max alpha |fv| |dP|)
    double forms[8];
    // Hartree / Hubbard forms: Haa Hab Hbb Uaa Uab Ubb
    double hforms[8];
    double Ein[4];     // Kinetic, Fock, Hartree, Hubbard of the current state
    double Eout[4];    // at the chosen step
    double E1tot, Ehtot, Etot_in, Etot_out;
    double step;
    double dn_max, dV_max, residual;
};

// Pulay / Anderson mixing (scf.cu)
constexpr int DIIS_MAX = 8;
struct DiisArgs {
    double2* P;            // state x (P_in), overwritten by the mixed state
    const double2* Pn;     // P_new
    float2* hist;          // slots x {dX, dR} x nn4 (complex64)
    float2* rprev;         // previous residual (complex64)
    size_t nn4;            // 4 N^2
    int slots[DIIS_MAX];   // history slots used
    double gamma[DIIS_MAX];
    int nslots, snew, spend;
    double beta;
    double* part;          // DIIS_CTAS x 2 x DIIS_MAX partial dots
};
}  // namespace forge
