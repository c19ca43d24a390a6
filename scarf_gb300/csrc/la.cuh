// Small dense linear algebra of the PCA eigensolver, written for this
// library (column-major storage, as the solver keeps its blocks):
//   gemm       C = alpha op(A) B + beta C, op(A) = A or A^T; SIMT tiles with
//              a deterministic split of K (partials reduced in a fixed order)
//   potrf      lower Cholesky factor of an m x m matrix (m <= 256), one CTA
//   trsm_rlt   Y <- Y L^-T for a lower L (the Cholesky-QR step), a thread per row
//   syev_f32   eigenvalues (ascending) and vectors of a symmetric m x m FP32
//              matrix (m <= 256, lower triangle read), one CTA running the
//              cyclic Jacobi method in parallel (round-robin) order
//   and vector helpers (symmetric matrix-vector product, rank-1 update,
//   Chebyshev recurrence step).
// Every routine runs on the caller's stream; scratch comes from the caller.
#pragma once

#include "common.cuh"

namespace sg {
namespace la {

// scratch elements of T that gemm needs for a split of K (0 when none)
size_t gemm_scratch(int m, int n, int k);

template <typename T>
int gemm(bool trans_a, int m, int n, int k, T alpha, const T* A, int lda, const T* B, int ldb, T beta, T* C, int ldc,
         T* scratch, cudaStream_t st);

// Lower Cholesky factor in place (the upper triangle is left as it was);
// *info (device) receives 0, or j + 1 when the j-th pivot is not positive.
template <typename T>
int potrf(int m, T* G, int ldg, int* info, cudaStream_t st);

// Y (n x m, ld n) <- Y L^-T with L the lower triangle of G (m x m, ld ldg)
template <typename T>
int trsm_rlt(int n, int m, const T* G, int ldg, T* Y, cudaStream_t st);

// Symmetric eigendecomposition: W ascending, V (m x m, ld m) the vectors in
// the same order; A is read (lower triangle) and left as it was. scratch:
// m * m floats when m > 192 (the vectors then live in global memory), else
// may be null. *info (device) receives 0, or -1 when the iteration did not
// converge.
int syev_f32(int m, const float* A, int lda, float* W, float* V, float* scratch, int* info, cudaStream_t st);

// y = alpha A x + beta y for a symmetric n x n A (column-major)
int symv_f32(int n, float alpha, const float* A, const float* x, float beta, float* y, cudaStream_t st);
// A_out = A - theta v v^T (n x n)
int syr_f32(int n, const float* A, float theta_neg, const float* v, float* A_out, cudaStream_t st);
// prev <- -prev - 2 cur (n elements): the Chebyshev recurrence's combination
int cheb_combine_f32(int64_t n, float* prev, const float* cur, cudaStream_t st);

}  // namespace la
}  // namespace sg
