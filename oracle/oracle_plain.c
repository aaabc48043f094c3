/* oracle_plain.c -- plain-loop CPU restatement of the reference's TSMTTSM / TSMM kernels.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  These loops are also the host C/OpenMP CPU
 * baseline: the same loop structure as the reference's test harness form.
 *
 * TSMTTSM follows GENV5 (tsmttsm/genv5.cuh:28-89, 9-26): every thread accumulates an M x N
 * partial in the working type over its own static chunk of K rows; the partials are summed in
 * fixed thread order (genv5.cuh:21-23) and C = beta*C + alpha*sum (genv5.cuh:25).
 * TSMM follows FIX3 (tsmm/fix3.cuh:20-38): one row at a time, sum_m A[r,m]*B[n,m] in the
 * working type, then C = beta*C + alpha*sum (axpby, cu_complex.h:164-169), or alpha*sum when
 * beta == 0 (BETAISZERO, fix3.cuh:31-32).  The row is read completely before it is written, so
 * A == C (in place, lda == ldc) is well defined.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

static int nthr(int n) {
#ifdef _OPENMP
  return n > 0 ? n : omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

#define DEF_TSMTTSM_REAL(NAME, T)                                                                  \
  void NAME(int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, const void* alpha_p,        \
            const T* B, int64_t ldb, const void* beta_p, T* C, int64_t ldc, int nthreads) {       \
    T alpha = *(const T*)alpha_p, beta = *(const T*)beta_p;                                        \
    int nt = nthr(nthreads);                                                                       \
    int64_t MN = M * N;                                                                            \
    T* part = (T*)calloc((size_t)nt * MN, sizeof(T));                                              \
    _Pragma("omp parallel num_threads(nt)") {                                                      \
      int t = 0, Tn = 1;                                                                           \
      PAR_IDS(t, Tn);                                                                              \
      int64_t k0 = K * t / Tn, k1 = K * (t + 1) / Tn;                                              \
      T* p = part + (size_t)t * MN;                                                                \
      for (int64_t k = k0; k < k1; k++) {                                                          \
        const T* a = A + k * lda;                                                                  \
        const T* b = B + k * ldb;                                                                  \
        for (int64_t n = 0; n < N; n++) {                                                          \
          T bv = b[n];                                                                             \
          T* pn = p + n * M;                                                                       \
          for (int64_t m = 0; m < M; m++) pn[m] += a[m] * bv;                                      \
        }                                                                                          \
      }                                                                                            \
    }                                                                                              \
    for (int64_t n = 0; n < N; n++)                                                                \
      for (int64_t m = 0; m < M; m++) {                                                            \
        T s = 0;                                                                                   \
        for (int t = 0; t < nt; t++) s += part[(size_t)t * MN + n * M + m];                        \
        T* out = &C[n * ldc + m];                                                                  \
        *out = (beta == 0) ? alpha * s : (*out) * beta + s * alpha;                                \
      }                                                                                            \
    free(part);                                                                                    \
  }

#define DEF_TSMTTSM_CPLX(NAME, T)                                                                  \
  void NAME(int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, const void* alpha_p,        \
            const T* B, int64_t ldb, const void* beta_p, T* C, int64_t ldc, int nthreads) {       \
    const T* al = (const T*)alpha_p;                                                               \
    const T* be = (const T*)beta_p;                                                                \
    int nt = nthr(nthreads);                                                                       \
    int64_t MN = M * N;                                                                            \
    T* part = (T*)calloc((size_t)nt * MN * 2, sizeof(T));                                          \
    _Pragma("omp parallel num_threads(nt)") {                                                      \
      int t = 0, Tn = 1;                                                                           \
      PAR_IDS(t, Tn);                                                                              \
      int64_t k0 = K * t / Tn, k1 = K * (t + 1) / Tn;                                              \
      T* p = part + (size_t)t * MN * 2;                                                            \
      for (int64_t k = k0; k < k1; k++) {                                                          \
        const T* a = A + 2 * k * lda;                                                              \
        const T* b = B + 2 * k * ldb;                                                              \
        for (int64_t n = 0; n < N; n++) {                                                          \
          T br = b[2 * n], bi = b[2 * n + 1];                                                      \
          T* pn = p + 2 * n * M;                                                                   \
          for (int64_t m = 0; m < M; m++) {                                                        \
            T ar = a[2 * m], ai = a[2 * m + 1];                                                    \
            pn[2 * m] += ar * br - ai * bi;                                                        \
            pn[2 * m + 1] += ar * bi + ai * br;                                                    \
          }                                                                                        \
        }                                                                                          \
      }                                                                                            \
    }                                                                                              \
    for (int64_t n = 0; n < N; n++)                                                                \
      for (int64_t m = 0; m < M; m++) {                                                            \
        T sr = 0, si = 0;                                                                          \
        for (int t = 0; t < nt; t++) {                                                             \
          sr += part[(size_t)t * MN * 2 + 2 * (n * M + m)];                                        \
          si += part[(size_t)t * MN * 2 + 2 * (n * M + m) + 1];                                    \
        }                                                                                          \
        T* out = &C[2 * (n * ldc + m)];                                                            \
        T rr = al[0] * sr - al[1] * si, ri = al[0] * si + al[1] * sr;                              \
        if (!(be[0] == 0 && be[1] == 0)) {                                                         \
          T cr = out[0], ci = out[1];                                                              \
          rr += be[0] * cr - be[1] * ci;                                                           \
          ri += be[0] * ci + be[1] * cr;                                                           \
        }                                                                                          \
        out[0] = rr;                                                                               \
        out[1] = ri;                                                                               \
      }                                                                                            \
    free(part);                                                                                    \
  }

#ifdef _OPENMP
#define PAR_IDS(t, Tn)             \
  do {                             \
    t = omp_get_thread_num();      \
    Tn = omp_get_num_threads();    \
  } while (0)
#else
#define PAR_IDS(t, Tn) \
  do {                 \
  } while (0)
#endif

DEF_TSMTTSM_REAL(orc_tsmttsm_s, float)
DEF_TSMTTSM_REAL(orc_tsmttsm_d, double)
DEF_TSMTTSM_CPLX(orc_tsmttsm_c, float)
DEF_TSMTTSM_CPLX(orc_tsmttsm_z, double)

#define DEF_TSMM_REAL(NAME, T)                                                                     \
  void NAME(int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, const void* alpha_p,        \
            const T* B, int64_t ldb, const void* beta_p, T* C, int64_t ldc, int nthreads) {       \
    T alpha = *(const T*)alpha_p, beta = *(const T*)beta_p;                                        \
    _Pragma("omp parallel num_threads(nthr(nthreads))") {                                          \
      T* tmp = (T*)malloc((size_t)(N > 0 ? N : 1) * sizeof(T));                                    \
      _Pragma("omp for schedule(static)") for (int64_t r = 0; r < K; r++) {                        \
        const T* a = A + r * lda;                                                                  \
        for (int64_t n = 0; n < N; n++) {                                                          \
          const T* b = B + n * ldb;                                                                \
          T s = 0;                                                                                 \
          for (int64_t m = 0; m < M; m++) s += a[m] * b[m];                                        \
          tmp[n] = s;                                                                              \
        }                                                                                          \
        T* c = C + r * ldc;                                                                        \
        for (int64_t n = 0; n < N; n++)                                                            \
          c[n] = (beta == 0) ? alpha * tmp[n] : beta * c[n] + alpha * tmp[n];                      \
      }                                                                                            \
      free(tmp);                                                                                   \
    }                                                                                              \
  }

#define DEF_TSMM_CPLX(NAME, T)                                                                     \
  void NAME(int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, const void* alpha_p,        \
            const T* B, int64_t ldb, const void* beta_p, T* C, int64_t ldc, int nthreads) {       \
    const T* al = (const T*)alpha_p;                                                               \
    const T* be = (const T*)beta_p;                                                                \
    int bz = (be[0] == 0 && be[1] == 0);                                                           \
    _Pragma("omp parallel num_threads(nthr(nthreads))") {                                          \
      T* tmp = (T*)malloc((size_t)(N > 0 ? N : 1) * 2 * sizeof(T));                                \
      _Pragma("omp for schedule(static)") for (int64_t r = 0; r < K; r++) {                        \
        const T* a = A + 2 * r * lda;                                                              \
        for (int64_t n = 0; n < N; n++) {                                                          \
          const T* b = B + 2 * n * ldb;                                                            \
          T sr = 0, si = 0;                                                                        \
          for (int64_t m = 0; m < M; m++) {                                                        \
            T ar = a[2 * m], ai = a[2 * m + 1], br = b[2 * m], bi = b[2 * m + 1];                  \
            sr += ar * br - ai * bi;                                                               \
            si += ar * bi + ai * br;                                                               \
          }                                                                                        \
          tmp[2 * n] = sr;                                                                         \
          tmp[2 * n + 1] = si;                                                                     \
        }                                                                                          \
        T* c = C + 2 * r * ldc;                                                                    \
        for (int64_t n = 0; n < N; n++) {                                                          \
          T sr = tmp[2 * n], si = tmp[2 * n + 1];                                                  \
          T rr = al[0] * sr - al[1] * si, ri = al[0] * si + al[1] * sr;                            \
          if (!bz) {                                                                               \
            T cr = c[2 * n], ci = c[2 * n + 1];                                                    \
            rr += be[0] * cr - be[1] * ci;                                                         \
            ri += be[0] * ci + be[1] * cr;                                                         \
          }                                                                                        \
          c[2 * n] = rr;                                                                           \
          c[2 * n + 1] = ri;                                                                       \
        }                                                                                          \
      }                                                                                            \
      free(tmp);                                                                                   \
    }                                                                                              \
  }

DEF_TSMM_REAL(orc_tsmm_s, float)
DEF_TSMM_REAL(orc_tsmm_d, double)
DEF_TSMM_CPLX(orc_tsmm_c, float)
DEF_TSMM_CPLX(orc_tsmm_z, double)
