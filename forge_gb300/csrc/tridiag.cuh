// Batched Householder reduction of Hermitian matrices (lower triangle) to real
// symmetric tridiagonal form, A = Q T Q^H, restating the blocked algorithm of
// LAPACK zhetrd/zlatrd (uplo = 'L') that the reference reaches through zheevr
// (LapackRoutines.f90:414-426).
//
// Per column (all k of the batch in one launch each):
//   trd_col   : update column col with the panel's previous reflectors, generate
//               the reflector (zlarfg) in the last CTA (deterministic partials);
//   trd_hemv  : y = A22 v over 64x64 tiles of the trailing lower triangle, every
//               element read once; row and column partials go to disjoint slots
//               (Yrow / Ycol) so the reduction order is fixed; extra CTAs form
//               the panel dots W^H v and V^H v;
//   trd_finish: y -= V s1 + W s2, W(:,i) = tau y, v written back, alpha2 in the last CTA;
//   trd_fix   : W(:,i) += alpha2 v.
// After each panel of NB columns, the trailing matrix gets A22 -= V W^H + W V^H
// (a rank-2k update on the GEMM engine of the chosen precision).
#pragma once
#include "cvec.cuh"
#include "forge_internal.cuh"

namespace forge {

constexpr int TRD_NB = 32;      // panel width
constexpr int TRD_TILE = 64;    // column granularity of the hemv partial slots (Yrow / Ycol)
constexpr int HV_RB = 64;       // hemv tile rows
constexpr int HV_CB = 64;       // hemv tile columns
constexpr int TRD_ROWS = 256;   // rows per CTA in the column kernels

template <class T>
struct TrdArgs {
    using V = typename CV<T>::type;
    V* A;
    int64_t lda, strideA, n;
    double* d;
    double* e;          // batch x n each
    V* tau;             // batch x n
    V* W;               // batch x (n x NB), ldw = n
    V* Yrow;            // batch x (nblk x n)
    V* Ycol;            // batch x (nblk x n)
    int64_t ystride;    // nblk * n
    V* Spart;           // batch x (nrb x 2NB)
    int64_t sstride;
    double* part;       // batch x pstride per-CTA partials
    int64_t pstride;
    double* scal;       // batch x 16
    unsigned* cnt;      // batch x 4
    // optional trailing-update override (the tensor-core rank-2k update of the mixed path):
    // A(p+w:n, p+w:n) -= V W^H + W V^H for the panel [p, p+w)
    int (*her2k)(cudaStream_t st, TrdArgs<T>& a, int64_t p, int64_t w, int64_t batch, void* user) = nullptr;
    void* her2k_user = nullptr;
};

template <class T>
int tridiagonalize(cudaStream_t st, TrdArgs<T>& a, int64_t batch);

}  // namespace forge
