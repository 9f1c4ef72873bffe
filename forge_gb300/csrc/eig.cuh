// Batched partial Hermitian eigen-solver: eigenpairs 1..iu of nb matrices
// (lower triangles, column-major), the operation of zdiagRed
// (LapackRoutines.f90:381-433) for every k point of a batch.
#pragma once
#include "forge_internal.cuh"
#include "tridiag.cuh"

namespace forge {

struct EigArgs {
    int64_t n, iu, batch;
    double2* A;                 // batch x (lda x n), overwritten by the reflectors
    int64_t lda, strideA;
    double2* X;                 // batch x (ldx x iu) eigenvectors
    int64_t ldx, strideX;
    double* w;                  // batch x iu eigenvalues (ascending)
    // workspace
    double *d, *e;              // batch x n
    double2* tau;               // batch x n
    double2* Wp;                // batch x n x NB (panel W)
    double2 *Yrow, *Ycol;       // batch x ystride
    int64_t ystride;
    double2* Spart;
    int64_t sstride;
    double* part;
    int64_t pstride;
    double* scal;               // batch x 16
    unsigned* cnt;              // batch x 4
    double* info;               // batch x 8
    int* clus;                  // batch x (iu + 2)
    double* Z;                  // batch x n x iu (row-major)
    double* scr;                // 4 x n x (scr_stride * batch)
    unsigned char* pivs;        // n x (scr_stride * batch)
    int64_t scr_stride;         // >= iu
    int* fail;                  // batch
    double2 *G, *T, *Wb, *W2b;  // back-transform: NB x NB, NB x NB, NB x iu, NB x iu per batch
    float* tf;                  // batch x 2n: FP32 copies of d and e^2 (FP32 bisection)
    double ortol_rel;
    int bisect_f32 = 0;         // 1: FP32 bisection first, FP64 bisection from its bracket
    int64_t iu_out = 0;         // mixed solver: FP64 columns written to X (0: all iu)
};

// workspace sizes (bytes) for a given problem
size_t eig_workspace_bytes(int64_t n, int64_t iu, int64_t batch);
// carve the workspace out of one device buffer
void eig_bind_workspace(EigArgs& g, void* base);

int eig_fp64(cudaStream_t st, EigArgs& g);
int tridiag_eigvecs(cudaStream_t st, EigArgs& g);
int backtransform_fp64(cudaStream_t st, const double2* A, int64_t lda, int64_t strideA, const double2* tau, int64_t n,
                       double2* X, int64_t ldx, int64_t strideX, int64_t iu, int64_t batch, double2* Gws,
                       double2* Tws, double2* Wws, double2* W2ws);

}  // namespace forge
