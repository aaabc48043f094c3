/* oracle.h -- CPU restatement of te42kyfo/skinny_matmul's tall-skinny products.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links or calls this code;
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use it,
 * and only as the reference results the GPU path is compared with (or as the timed CPU
 * implementation of the reference's loops).
 *
 * Three families:
 *   orc_tsmttsm_* / orc_tsmm_*   plain loops in the working type, OpenMP-parallel in the
 *                                shape of the reference harness (per-thread partials over a
 *                                static K chunk, reduced in fixed thread order).
 *   orc_tsmttsm_pq               double inputs, double-double ("PseudoQuad") accumulation,
 *                                restating PseudoQuad.cuh:10-31,66-75,96-108,137-152.
 *   orc_*_exact_*                exact super-accumulator ground truth, returned as a
 *                                correctly rounded double-double (hi, lo).
 *
 * Layouts (reference semantics, versions.hpp:43-45):
 *   TSMTTSM  C[n*ldc+m]   = alpha * sum_k A[k*lda+m] * B[k*ldb+n] + beta * C[n*ldc+m]
 *   TSMM     C[r*ldc+n]   = alpha * sum_m A[r*lda+m] * B[n*ldb+m] + beta * C[r*ldc+n]
 *   Complex values are interleaved (re, im); products use the plain transpose (no conjugate),
 *   as the reference's cuBLAS oracle does (tsmttsm/gen_cublas.cuh:29-39, OP_T).
 *   beta == 0 means C is not read (BLAS convention, tsmm/fix3.cuh:31-35 BETAISZERO).
 *   TSMM with A == C (and lda == ldc) is the in-place form: every output row is computed from
 *   the row's old contents before it is overwritten.
 * alpha/beta point to one value of the working type (two doubles/floats for complex).
 */
#ifndef SKINNY_ORACLE_H
#define SKINNY_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

void orc_tsmttsm_s(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const void* alpha,
                   const float* B, int64_t ldb, const void* beta, float* C, int64_t ldc, int nthreads);
void orc_tsmttsm_d(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const void* alpha,
                   const double* B, int64_t ldb, const void* beta, double* C, int64_t ldc, int nthreads);
void orc_tsmttsm_c(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const void* alpha,
                   const float* B, int64_t ldb, const void* beta, float* C, int64_t ldc, int nthreads);
void orc_tsmttsm_z(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const void* alpha,
                   const double* B, int64_t ldb, const void* beta, double* C, int64_t ldc, int nthreads);
void orc_tsmttsm_pq(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const void* alpha,
                    const double* B, int64_t ldb, const void* beta, double* C, int64_t ldc, int nthreads);

void orc_tsmm_s(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const void* alpha,
                const float* B, int64_t ldb, const void* beta, float* C, int64_t ldc, int nthreads);
void orc_tsmm_d(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const void* alpha,
                const double* B, int64_t ldb, const void* beta, double* C, int64_t ldc, int nthreads);
void orc_tsmm_c(int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const void* alpha,
                const float* B, int64_t ldb, const void* beta, float* C, int64_t ldc, int nthreads);
void orc_tsmm_z(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const void* alpha,
                const double* B, int64_t ldb, const void* beta, double* C, int64_t ldc, int nthreads);

/* Exact S = A^T B (TSMTTSM) or S = A B (TSMM) for double inputs (float inputs convert exactly),
 * rounded once to a double-double: S = hi + lo with |S - hi - lo| <= ulp(lo)/2.
 * Real: hi/lo have the C layout above (lds = ldc).  Complex (_z): hi/lo are interleaved. */
void orc_tsmttsm_exact_d(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                         const double* B, int64_t ldb, double* hi, double* lo, int64_t lds, int nthreads);
void orc_tsmttsm_exact_z(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                         const double* B, int64_t ldb, double* hi, double* lo, int64_t lds, int nthreads);
void orc_tsmm_exact_d(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                      const double* B, int64_t ldb, double* hi, double* lo, int64_t lds, int nthreads);
void orc_tsmm_exact_z(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                      const double* B, int64_t ldb, double* hi, double* lo, int64_t lds, int nthreads);

/* Exact dot product of two double vectors (strided), rounded to double-double. */
void orc_dot_exact(int64_t K, const double* a, int64_t inca, const double* b, int64_t incb,
                   double* hi, double* lo);

/* PseudoQuad primitives exposed for unit tests (PseudoQuad.cuh:10-31,66-75,96-108,137-152). */
void orc_pq_fast2sum(double a, double b, double* s, double* t);
void orc_pq_gen2sum(double a, double b, double* s, double* t);
void orc_pq_fma2mult(double a, double b, double* s, double* t);
void orc_pq_accu(double xs, double xt, double ys, double yt, double* s, double* t);
void orc_pq_axpy2(double cs, double ct, double a, double b, double* s, double* t);
void orc_pq_scale2(double as, double at, double b, double* s, double* t);

int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
