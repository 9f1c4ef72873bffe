// Internal declarations shared by the forge_gpu translation units.
//
// Device layout (all arrays column-major like the reference's Fortran arrays):
//   coords      N x 3 FP64                  Coords(i,:)            (Main.f90:82)
//   tab_t[7]    N x N FP64 each: t0, tm1..3, tp1..3 = ft(r_i, r_j -/+ R_c)
//   tab_v[10]   N x N FP64 each: v0, vm1..3, vp1..3 = fv(r_i, r_j -/+ R_c),
//               vt1..3 = fv(r_j, r_i - R_c)  (the transposed call of HartreeFock.f90:110)
//   LR          N x N FP64                  LongRange              (HartreeFock.f90:14)
//   P, P_in     4 x N x N complex128        zFock / zFockIn        (Main.f90:105-106)
//   H           Nk x N x N complex128       H(k), lower triangle   (HartreeFock.f90:416)
//   X           Nk x N x nUpper complex128  eigenvectors 1..nUpper (LapackRoutines.f90:428)
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/forge_gpu.h"
#include "profiler.cuh"

namespace forge {

// ---------------------------------------------------------------- complex helpers
struct cplx {
    double re, im;
};

__host__ __device__ inline double2 cmake(double r, double i) { return make_double2(r, i); }
__host__ __device__ inline double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__host__ __device__ inline double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__host__ __device__ inline double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__host__ __device__ inline double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// a * conj(b)
__host__ __device__ inline double2 cmulc(double2 a, double2 b) {
    return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// conj(a) * b
__host__ __device__ inline double2 cjmul(double2 a, double2 b) {
    return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__host__ __device__ inline double cabs2(double2 a) { return a.x * a.x + a.y * a.y; }

// ---------------------------------------------------------------- error plumbing
struct Status {
    int code = 0;
    std::string msg;
};

void set_error(int code, const char* fmt, ...);
int last_error_code();

#define FORGE_CUDA(call)                                                                        \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            ::forge::set_error(FORGE_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,       \
                               cudaGetErrorString(e_));                                         \
            return FORGE_ERR_CUDA;                                                              \
        }                                                                                       \
    } while (0)

// every kernel launch site ends with FORGE_LAUNCH_CHECK(), which also counts the launch
void count_launch();

#define FORGE_LAUNCH_CHECK()                                                                    \
    do {                                                                                        \
        ::forge::count_launch();                                                                \
        cudaError_t e_ = cudaGetLastError();                                                    \
        if (e_ != cudaSuccess) {                                                                \
            ::forge::set_error(FORGE_ERR_CUDA, "%s:%d launch: %s", __FILE__, __LINE__,          \
                               cudaGetErrorString(e_));                                         \
            return FORGE_ERR_CUDA;                                                              \
        }                                                                                       \
    } while (0)

#define FORGE_TRY(expr)                   \
    do {                                  \
        int rc_ = (expr);                 \
        if (rc_ != 0) return rc_;         \
    } while (0)

// ---------------------------------------------------------------- device workspace
// Simple growable device buffers owned by a context.
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    int ensure(size_t nbytes);
    void release();
    template <class T>
    T* as() const { return static_cast<T*>(ptr); }
};

// Eigen-solver workspace for a batch of k points.
struct EigWork {
    DevBuf d, e, tau;          // tridiagonal (batch x N), (batch x N), tau (batch x N complex)
    DevBuf W;                  // latrd panel W: batch x N x nb complex
    DevBuf vbuf, ybuf;         // per-column vectors: batch x N complex
    DevBuf scal;               // per-k scalars (batch x 16 doubles)
    DevBuf counters;           // per-k block counters (batch x 8 uint32)
    DevBuf small;              // per-k small vectors (batch x 4*nb complex)
    DevBuf w;                  // eigenvalues batch x nUpper (FP64)
    DevBuf Z;                  // real tridiagonal eigenvectors, batch x N x nUpper
    DevBuf lu;                 // inverse-iteration LU scratch
    DevBuf Tw;                 // compact-WY T factors, batch x nb x nb complex
    DevBuf Wbt;                // back-transform workspace: batch x nb x m complex
    DevBuf clus;               // cluster bookkeeping (int)
};

struct Context {
    forge_setup s;
    int64_t N = 0, Nk = 0, nnc = 0, nLower = 0, nUpper = 0, numb = 0, NP = 0;
    double t1[2], t2[2];
    std::vector<int64_t> ucell1, ucell2, kcomp;   // kcomp: Nk x 2 (column-major, like the reference)
    std::vector<double> kvals;                   // numk x numk x 2 (column-major)
    std::vector<double> coords_h;                // N x 3 column-major

    cudaStream_t stream = nullptr;

    // geometry / tables
    DevBuf coords, tab_t, tab_v, LR;
    bool tables_ready = false, lr_ready = false;
    // state
    DevBuf P, P_in, P_new, bulk, V, dens, dens_in, V_old;
    // per-iteration outputs
    DevBuf H, X, bands, evals;
    DevBuf kvecs;                                // Nk x 2 k vectors (flat k order)
    DevBuf kphase;                               // Nk x nnc complex: exp(-i k.R_c) (float dot, HartreeFock.f90:90)
    DevBuf bphase;                               // Nk x nnc complex: integer Bloch phase (HartreeFock.f90:471)
    DevBuf sort_idx, sort_e;                     // sorted window states
    DevBuf red;                                  // reduction scratch
    DevBuf scalars;                              // device-side scalars (Fermi level, energies, step)
    EigWork ew;
    int64_t eig_batch = 0;                       // k points per eigen-solver batch
    int info = 0;                                // last eigen-solver info
    int precision = FORGE_PREC_FP64;
    bool refined = false;                        // the last solve's eigenpairs were refined to FP64 accuracy
};

// ---------------------------------------------------------------- kernels (host launchers)
int launch_pair_tables(Context& c);
int launch_long_range(Context& c);
int launch_assemble(Context& c, const double* dV, const double2* dP, int64_t k0, int64_t nk, double2* dH);
int eig_fp64_batch(Context& c, double2* H, int64_t nb_k, double* w_out, double2* X_out, int64_t ldx, int* info);
int launch_bulk_projector(Context& c, const double2* X, int64_t k0, int64_t nk, double2* bulk, bool first);
int launch_window_projector(Context& c, const int64_t* d_states, int64_t nocc, int64_t npart, double2 zdeg,
                            double2* P);
int launch_scale_combine(Context& c, const double2* bulk, double2* P);
int launch_energies(Context& c, const double2* Pa, const double2* Pb, const double* da, const double* db,
                    double* out /* device: 16 doubles */);
int launch_potential(Context& c, const double* dens, double* V);
int launch_mix(Context& c, double step, double2* P, const double2* P_new, const double2* P_in, double* dens,
               const double* dens_in, double* out);

// C3-reduced solve (c3.cu)
struct C3Tables {
    std::vector<int64_t> reps;      // 0-based k of the first point of each C3 orbit
    int64_t nslots = 0;             // eigenvector slots: Nk, plus two per C3-invariant k
    std::vector<int64_t> slot_tab;  // per slot: representative index, rotation (0 none, 1 nC3pairs, 2 twice)
    std::vector<int64_t> extra;     // per k: its first extra slot (invariant k) or -1
    std::vector<double2> phase;     // per slot: the N site phases of the rotation
};
bool c3_invariant(int64_t numk, int64_t k);
int c3_build_tables(int64_t numk, int64_t N, int64_t nlayers, const int64_t* kcomp, const int64_t* RotateLayers,
                    C3Tables& t);
int launch_c3_rotate(cudaStream_t st, const double2* Xr, const double* wr, int64_t N, int64_t iu, int64_t nslots,
                     const int64_t* slot_tab, const int64_t* perm, const double2* phase, double2* X, double* w);

// valley projection (valley.cu)
struct ValleyTerms {
    std::vector<int64_t> rowp, col;  // CSR rows of V(k) (N + 1) and column of each term
    std::vector<double> coef;        // sign(cos 3 phi) / sqrt(27); the term is i coef phase
    std::vector<int> code;           // phase: 0 home cell, c = 1..3 exp(-i k.R_c), 3 + c exp(+i k.R_c)
};
int valley_build_terms(const Context& c, const int64_t* RotateLayers, ValleyTerms& t);
void valley_phases(const Context& c, std::vector<double2>& ph);
int launch_valley_gram(cudaStream_t st, const double2* X, int64_t N, int64_t iu, int64_t c0, int64_t nb, int64_t Nk,
                       const int64_t* rowp, const int64_t* col, const double* coef, const int* code,
                       const double2* ph, double2* W, double2* G);
int launch_valley_rotate(cudaStream_t st, const double2* X, int64_t N, int64_t iu, int64_t c0, int64_t nb, int64_t Nk,
                         const double2* S, double2* Xv);
int rr_small(int n, const double2* G, const double2* S, double* theta, double2* M);

// symmetry switches of the SCF loop (symmetry.cu)
int launch_symmetrize(cudaStream_t st, double2* P, double2* scratch, const int64_t* perm, int64_t N, bool T, bool C2,
                      bool C2T);
// order parameters of P(0): nblocks x 4 partial sums (layer, sublattice, |P - C2T P|^2, |P - C3 P|^2)
int launch_order_params(cudaStream_t st, const double2* P0, int64_t N, int64_t L, const int64_t* c2,
                        const int64_t* c3, double* part, int nblocks);

// device helpers shared across units
__device__ double dev_ft(const forge_setup& s, double xi, double yi, double zi, double xj, double yj, double zj);
__device__ double dev_fv(const forge_setup& s, double xi, double yi, double zi, double xj, double yj, double zj);

}  // namespace forge
