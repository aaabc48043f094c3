// tsmm.cuh -- TSMM on CUDA cores: C(KxN) = alpha * A(KxM) B(MxN) + beta * C, C may be A.
//
// Replaces the reference's tsmm/fix{1,2,3,4}, fix_fb, var1, varip{1,2,3}, fix_ip_ghost and
// var_ip_ghost kernels (tsmm/fix3.cuh:4-65, fix_fb.cuh:5-102, fix_ip_ghost.cuh:4-44 ...).
// Same layouts: A[r*lda+m], B[n*ldb+m] (column n contiguous over m), C[r*ldc+n].
//
// Design:
//   * B is staged once per CTA in shared memory as Bs[m][n] (n fastest), so a thread reads the
//     TN consecutive columns it owns for each m without bank conflicts.
//   * A thread owns one row and TN consecutive output columns (a "cell"); the gn cells of a row
//     are consecutive lanes of one warp (gn is a power of two <= 32), so each row's outputs are
//     written as one contiguous, coalesced run.
//   * In place (A == C, lda == ldc): every lane finishes reading its row of A before the warp
//     passes __syncwarp(), and only then are outputs written; rows never cross warps, so no
//     output can overwrite input that another thread still needs.  beta*C reads the element the
//     same thread then overwrites.
//   * In place with M == N (and accumulation in the working type), beta is folded into B's diagonal
//     while B is staged: C = A (alpha B + beta I), so the epilogue neither reads C nor runs the
//     beta FMA on the FP64 pipe.
//   * Rows are distributed grid-stride over a persistent grid, U rows per thread and step (U = 4
//     for narrow widths so that enough loads are in flight to stream at HBM speed); all lanes of
//     a warp run the same trip count so the __syncwarp() is always reached by the full warp.
#pragma once
#include "common.cuh"
#include "tsmttsm.cuh"  // tzero

namespace skinny {

template <typename T>
struct TsmmArgs {
  const T* A;
  const T* B;
  T* C;
  int64_t K, lda, ldb, ldc;
  int M, N;
  T alpha, beta;
  int beta_zero;
  int fold;  // Bs = alpha B + beta I (in place, M == N); the epilogue then writes the sums as they are
  int gn;  // cells per row (power of two, <= 32)
  int np;  // padded width of Bs (gn * TN)
};

constexpr int TSMM_THREADS = 256;

template <typename T, typename Acc, int TN, int U>
__global__ void __launch_bounds__(TSMM_THREADS) tsmm_kernel(const TsmmArgs<T> p) {
  typedef Ops<T, Acc> O;
  constexpr int NT = TSMM_THREADS;
  extern __shared__ __align__(128) unsigned char smem[];
  T* Bs = reinterpret_cast<T*>(smem);
  const int M = p.M, N = p.N, np = p.np, gn = p.gn;
  const bool fold = p.fold != 0;
  for (int e = threadIdx.x; e < M * np; e += NT) {
    int m = e / np, n = e - m * np;
    const T b = (n < N) ? p.B[(int64_t)n * p.ldb + m] : tzero<T>();
    if constexpr (sizeof(Acc) == sizeof(T)) {
      Bs[e] = (fold && n < N) ? fold_entry(p.alpha, b, p.beta, m == n) : b;
    } else {
      Bs[e] = b;
    }
  }
  __syncthreads();

  // U rows per thread and step (r = base + j*RS + rs): for narrow products the loads of U rows
  // are in flight together, which a streaming (HBM-bound) width needs
  const int RS = NT / gn;  // rows per CTA step and unit (gn divides 32, so NT % gn == 0)
  const int cell = threadIdx.x % gn, rs = threadIdx.x / gn;
  const int n0 = cell * TN;
  const int64_t step = (int64_t)gridDim.x * RS * U;
  const bool alpha_one = fold || O::is_one(p.alpha), bz = fold || p.beta_zero != 0;  // decided once
  for (int64_t base = (int64_t)blockIdx.x * RS * U; base < p.K; base += step) {
    bool valid[U];
#pragma unroll
    for (int j = 0; j < U; j++) valid[j] = base + (int64_t)j * RS + rs < p.K;
    Acc acc[U][TN];
#pragma unroll
    for (int j = 0; j < U; j++)
#pragma unroll
      for (int u = 0; u < TN; u++) acc[j][u] = O::zero();
#pragma unroll 4
    for (int m = 0; m < M; m++) {
      T a[U];
#pragma unroll
      for (int j = 0; j < U; j++) a[j] = valid[j] ? p.A[(base + (int64_t)j * RS + rs) * p.lda + m] : tzero<T>();
      const T* b = Bs + m * np + n0;
#pragma unroll
      for (int j = 0; j < U; j++)
#pragma unroll
        for (int u = 0; u < TN; u++) acc[j][u] = O::mac(acc[j][u], a[j], b[u]);
    }
    __syncwarp();  // the whole rows have been read before any of them is overwritten (in place)
    T cv[U][TN];
    if (!bz) {  // C values of all U rows in flight together
#pragma unroll
      for (int j = 0; j < U; j++)
#pragma unroll
        for (int u = 0; u < TN; u++)
          cv[j][u] = (valid[j] && n0 + u < N) ? p.C[(base + (int64_t)j * RS + rs) * p.ldc + n0 + u] : tzero<T>();
    }
#pragma unroll
    for (int j = 0; j < U; j++) {
      if (!valid[j]) continue;
      T* c_row = p.C + (base + (int64_t)j * RS + rs) * p.ldc;
#pragma unroll
      for (int u = 0; u < TN; u++) {
        const int n = n0 + u;
        if (n < N)
          c_row[n] = alpha_one ? O::finish1(acc[j][u], p.beta, bz, &cv[j][u])
                               : O::finish(acc[j][u], p.alpha, p.beta, bz, &cv[j][u]);
      }
    }
  }
}

}  // namespace skinny
