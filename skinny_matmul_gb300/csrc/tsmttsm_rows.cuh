// tsmttsm_rows.cuh -- TSMTTSM on CUDA cores for narrow products (padded M x N up to 16 entries, or
// 8 x 8 in FP64): C(MxN) = alpha * A^T B + beta * C.
//
// Replaces, for these widths, the reference's GENV3X / SPECSMALL blockProductKernel +
// deviceReduce pairs (tsmttsm/genv3x.cuh:29-81, specsmall.cuh:28-90), which on GB300 stream
// narrow products faster than the tiled ring kernel (tsmttsm.cuh) because every warp reads
// global memory directly and many warps per SM keep loads in flight.  Same layouts:
//   A: K x M row-major (A[k*lda+m]), B: K x N row-major (B[k*ldb+n]), C[n*ldc+m].
//
// Design (one launch, no separate reduction kernel):
//   * A thread owns whole rows: U rows per step, NT rows apart (consecutive threads read
//     consecutive rows, so every load instruction of a warp is one coalesced run), and keeps the
//     full TM x TN register tile of partial sums; FP64 rows are read as 16-byte pairs where the
//     leading dimensions allow it.  Gram mode (A == B) reads A only.
//   * Rows are spread grid-stride over a grid of several CTAs per SM; no shared-memory staging,
//     no barriers in the streaming loop.
//   * Reduction: butterfly warp shuffles, the warps of a CTA in warp order through shared memory,
//     one partial per CTA in the workspace, and the last CTA to take the ticket sums the CTA
//     partials in CTA order (slices of the CTA range, then the slices in order) and applies
//     alpha / beta.  The result is deterministic; the ticket is reset for the next launch.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "tsmttsm.cuh"

namespace skinny {

constexpr int ROWS_THREADS = 256;

template <typename T>
struct RowsArgs {
  const T* A;
  const T* B;
  T* C;
  int64_t K, lda, ldb, ldc;
  int M, N;
  T alpha, beta;
  int beta_zero, gram;
  int vec_a, vec_b;  // FP64 rows read as 16-byte pairs (aligned base, even ld >= the padded width)
  void* partials;
  unsigned* counter;
};

// W values of one row (zero beyond n or for a row past the end)
template <typename T, int W>
__device__ __forceinline__ void row_vals(const T* __restrict__ row, int n, bool ok, bool vec, T (&v)[W]) {
  if constexpr (std::is_same<T, double>::value && W >= 2) {
    if (vec) {
#pragma unroll
      for (int x = 0; x < W; x += 2) {
        const double2 d = ok ? __ldg(reinterpret_cast<const double2*>(row + x)) : make_double2(0.0, 0.0);
        v[x] = x < n ? d.x : 0.0;
        v[x + 1] = x + 1 < n ? d.y : 0.0;
      }
      return;
    }
  }
#pragma unroll
  for (int x = 0; x < W; x++) v[x] = (ok && x < n) ? row[x] : tzero<T>();
}

template <typename T, typename Acc, int TM, int TN, int U>
__global__ void __launch_bounds__(ROWS_THREADS) tsmttsm_rows_kernel(const RowsArgs<T> p) {
  typedef Ops<T, Acc> O;
  constexpr int NT = ROWS_THREADS, NW = NT / 32, TMN = TM * TN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int M = p.M, N = p.N;
  const bool gram = p.gram != 0;

  Acc acc[TM][TN];
#pragma unroll
  for (int x = 0; x < TM; x++)
#pragma unroll
    for (int y = 0; y < TN; y++) acc[x][y] = O::zero();

  const int64_t stride = (int64_t)gridDim.x * NT * U;
  for (int64_t base = (int64_t)blockIdx.x * NT * U + tid; base < p.K; base += stride) {
    T a[U][TM], b[U][TN];
#pragma unroll
    for (int j = 0; j < U; j++) {
      const int64_t r = base + (int64_t)j * NT;
      const bool ok = r < p.K;
      row_vals<T, TM>(p.A + (ok ? r : 0) * p.lda, M, ok, p.vec_a != 0, a[j]);
      if (!gram) row_vals<T, TN>(p.B + (ok ? r : 0) * p.ldb, N, ok, p.vec_b != 0, b[j]);
    }
#pragma unroll
    for (int j = 0; j < U; j++)
#pragma unroll
      for (int x = 0; x < TM; x++)
#pragma unroll
        for (int y = 0; y < TN; y++) {
          T bv;
          if constexpr (TN <= TM) {
            bv = gram ? a[j][y] : b[j][y];
          } else {
            bv = b[j][y];  // Gram mode is never planned with TN > TM
          }
          acc[x][y] = O::mac(acc[x][y], a[j][x], bv);
        }
  }

  // ---- CTA reduction: warp butterflies, then the warps in order ------------------------------
#pragma unroll
  for (int x = 0; x < TM; x++)
#pragma unroll
    for (int y = 0; y < TN; y++)
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) acc[x][y] = O::add(acc[x][y], O::shfl_xor(acc[x][y], o));
  __shared__ Acc wsum[NW][TMN];
  __shared__ Acc slices[NT];
  __shared__ int s_last;
  if (lane == 0) {
#pragma unroll
    for (int x = 0; x < TM; x++)
#pragma unroll
      for (int y = 0; y < TN; y++) wsum[warp][y * TM + x] = acc[x][y];
  }
  __syncthreads();
  const int MN = M * N;
  Acc* part = reinterpret_cast<Acc*>(p.partials);
  if (tid < MN) {
    const int m = tid % M, n = tid / M;
    Acc s = wsum[0][n * TM + m];
#pragma unroll
    for (int w = 1; w < NW; w++) s = O::add(s, wsum[w][n * TM + m]);
    part[(size_t)blockIdx.x * MN + tid] = s;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(p.counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();

  // ---- last CTA: the CTA partials in CTA order (P slices of the CTA range, then the slices) ---
  const int nb = gridDim.x;
  const int P = NT / MN;  // MN <= 64, so P >= 4
  const int e = tid % MN, j = tid / MN;
  if (j < P) {
    Acc sum = O::zero();
    const int b0 = (int)((int64_t)nb * j / P), b1 = (int)((int64_t)nb * (j + 1) / P);
    for (int b = b0; b < b1; b++) sum = O::add(sum, ldcg(&part[(size_t)b * MN + e]));
    slices[j * MN + e] = sum;
  }
  __syncthreads();
  if (tid < MN) {
    Acc s = slices[tid];
    for (int q = 1; q < P; q++) s = O::add(s, slices[q * MN + tid]);
    const int m = tid % M, n = tid / M;
    T* c = p.C + (int64_t)n * p.ldc + m;
    *c = O::finish(s, p.alpha, p.beta, p.beta_zero != 0, c);
  }
  if (tid == 0) *p.counter = 0u;
}

}  // namespace skinny
