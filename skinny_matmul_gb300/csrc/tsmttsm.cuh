// tsmttsm.cuh -- TSMTTSM on CUDA cores: C(MxN) = alpha * A^T B + beta * C.
//
// Replaces the reference's GENV{3,3X,5,6,7,8}/SPECSMALL blockProductKernel + deviceReduce pairs
// (tsmttsm/genv5.cuh:9-114, genv7.cuh:10-154, specsmall.cuh:10-125).  Same layouts:
//   A: K x M row-major (A[k*lda+m]), B: K x N row-major (B[k*ldb+n]), C[n*ldc+m].
//
// Design (one persistent launch, no second reduce kernel):
//   * The K rows are cut into tiles of R rows; each CTA owns a contiguous run of tiles.
//   * Full tiles stream global -> shared with 1-D TMA bulk copies (cp.async.bulk) into a ring
//     of `stages` buffers, completion tracked by mbarriers (bounded waits, no trap).  The last
//     tile of the matrix (which may be short, and whose last row may end the allocation) and
//     unaligned operands use plain coalesced loads instead.
//   * Every thread owns a TM x TN register tile of partial sums for a fixed (m, n) block and a
//     fixed row slice; rows are read from shared memory.
//   * Gram mode (A == B, lda == ldb, M == N) copies only A (reference SELF mode, genv7.cuh:139).
//   * Partials are reduced within the CTA (warp shuffles, then fixed-order shared-memory phases),
//     written to a workspace, and the last CTA to take a ticket (atomicAdd) sums all CTA
//     partials in CTA order and applies alpha/beta.  The result is deterministic and the
//     ticket counter is reset to 0 for the next launch.
#pragma once
#include "common.cuh"

namespace skinny {

template <typename T>
struct TsmttsmArgs {
  const T* A;
  const T* B;
  T* C;
  int64_t K, lda, ldb, ldc;
  int64_t lda_s, ldb_s;  // row strides of the shared tiles (= lda/ldb when bulk, else M/N)
  int M, N;
  T alpha, beta;
  int beta_zero, gram, bulk;
  int rows;    // rows per tile (multiple of 16)
  int stages;  // ring depth
  int64_t ntiles;
  uint32_t bytes_a, bytes_b;  // shared bytes per stage for A and B (multiples of 128)
  uint32_t smem_avail;         // dynamic shared bytes after the header
  void* partials;
  unsigned* counter;
  int* err;
  uint32_t polls;  // poll limit of the bounded waits on the copy ring
};

template <typename T>
__device__ __forceinline__ T tzero() {
  return T(0);
}
template <>
__device__ __forceinline__ c32 tzero<c32>() {
  return {0.f, 0.f};
}
template <>
__device__ __forceinline__ c64 tzero<c64>() {
  return {0.0, 0.0};
}
template <>
__device__ __forceinline__ c32h tzero<c32h>() {
  return {0.f, 0.f};
}
template <>
__device__ __forceinline__ c64h tzero<c64h>() {
  return {0.0, 0.0};
}

// L2-coherent loads of partials written by other CTAs (L1 is not coherent across SMs).
__device__ __forceinline__ float ldcg(const float* p) { return __ldcg(p); }
__device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ c32 ldcg(const c32* p) {
  float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return {v.x, v.y};
}
__device__ __forceinline__ c64 ldcg(const c64* p) {
  double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return {v.x, v.y};
}
__device__ __forceinline__ c32h ldcg(const c32h* p) {
  float2 v = __ldcg(reinterpret_cast<const float2*>(p));
  return {v.x, v.y};
}
__device__ __forceinline__ c64h ldcg(const c64h* p) {
  double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return {v.x, v.y};
}
__device__ __forceinline__ dd ldcg(const dd* p) {
  double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  return {v.x, v.y};
}
__device__ __forceinline__ zdd ldcg(const zdd* p) {
  const double2 a = __ldcg(reinterpret_cast<const double2*>(p)), b = __ldcg(reinterpret_cast<const double2*>(p) + 1);
  return {{a.x, a.y}, {b.x, b.y}};
}

constexpr int TSMTTSM_THREADS = 256;
constexpr int SMEM_HEADER = 128;  // mbarriers live here

template <typename T, typename Acc, int TM, int TN>
__global__ void __launch_bounds__(TSMTTSM_THREADS, 1) tsmttsm_kernel(const TsmttsmArgs<T> p) {
  typedef Ops<T, Acc> O;
  constexpr int NT = TSMTTSM_THREADS;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);

  const int tid = threadIdx.x;
  const int M = p.M, N = p.N;
  const int gm = ceil_div(M, TM), gn = ceil_div(N, TN);
  // Cells (TM x TN blocks of C) are split into groups of <= NT along gridDim.y; every group
  // streams all rows and owns a disjoint set of C entries.
  const int cbase = blockIdx.y * NT;
  const int G = min(NT, gm * gn - cbase);  // thread cells of this group per row slice
  const int RS = NT / G;                    // row slices
  const int cell = cbase + tid % G, rs = tid / G;
  const bool active = rs < RS;
  const int m0 = (cell % gm) * TM, n0 = (cell / gm) * TN;

  const int64_t t_begin = p.ntiles * blockIdx.x / gridDim.x;
  const int64_t t_end = p.ntiles * (blockIdx.x + 1) / gridDim.x;
  const int nt = (int)(t_end - t_begin);
  const int64_t ldb_s = p.gram ? p.lda_s : p.ldb_s;
  const uint32_t stage_bytes = p.bytes_a + p.bytes_b;

  auto stage_a = [&](int s) { return reinterpret_cast<T*>(smem + SMEM_HEADER + (size_t)s * stage_bytes); };
  auto stage_b = [&](int s) {
    return p.gram ? stage_a(s) : reinterpret_cast<T*>(smem + SMEM_HEADER + (size_t)s * stage_bytes + p.bytes_a);
  };
  // A tile is bulk-loadable if its byte range ends before the last row starts.
  auto is_bulk = [&](int64_t t) { return p.bulk && (t + 1) * (int64_t)p.rows < p.K; };
  auto issue = [&](int64_t t, int s) {
    const int64_t r0 = t * p.rows;
    const uint32_t ba = (uint32_t)(p.rows * p.lda * (int64_t)sizeof(T));
    const uint32_t bb = p.gram ? 0u : (uint32_t)(p.rows * p.ldb * (int64_t)sizeof(T));
    mbar_arrive_expect_tx(&bars[s], ba + bb);
    bulk_g2s(stage_a(s), p.A + r0 * p.lda, ba, &bars[s]);
    if (!p.gram) bulk_g2s(stage_b(s), p.B + r0 * p.ldb, bb, &bars[s]);
  };

  if (p.bulk && tid == 0) {
    for (int s = 0; s < p.stages; s++) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (p.bulk && tid == 0) {
    for (int i = 0; i < nt && i < p.stages; i++)
      if (is_bulk(t_begin + i)) issue(t_begin + i, i);
  }

  Acc acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) acc[i][j] = O::zero();

  int bail = -1;  // ring position whose wait gave up
  for (int i = 0; i < nt; i++) {
    const int64_t t = t_begin + i;
    const int s = i % p.stages;
    const int64_t r0 = t * p.rows;
    const int rows = (int)((p.K - r0) < p.rows ? (p.K - r0) : p.rows);
    T* As = stage_a(s);
    T* Bs = stage_b(s);
    if (is_bulk(t)) {
      bool ok = mbar_wait_bounded(&bars[s], (uint32_t)((i / p.stages) & 1), p.err, p.polls);
      if (__syncthreads_or(!ok)) {
        bail = i;
        break;
      }
    } else {
      // plain coalesced loads of columns [0, M) / [0, N) of `rows` rows, ld layout kept
      for (int e = tid; e < rows * M; e += NT) {
        int r = e / M, m = e - r * M;
        As[r * p.lda_s + m] = p.A[(r0 + r) * p.lda + m];
      }
      if (!p.gram)
        for (int e = tid; e < rows * N; e += NT) {
          int r = e / N, n = e - r * N;
          Bs[r * p.ldb_s + n] = p.B[(r0 + r) * p.ldb + n];
        }
      __syncthreads();
    }
    if (active) {
      for (int r = rs; r < rows; r += RS) {
        T a[TM], b[TN];
#pragma unroll
        for (int x = 0; x < TM; x++) a[x] = (m0 + x < M) ? As[r * p.lda_s + m0 + x] : tzero<T>();
#pragma unroll
        for (int y = 0; y < TN; y++) b[y] = (n0 + y < N) ? Bs[r * ldb_s + n0 + y] : tzero<T>();
#pragma unroll
        for (int x = 0; x < TM; x++)
#pragma unroll
          for (int y = 0; y < TN; y++) acc[x][y] = O::mac(acc[x][y], a[x], b[y]);
      }
    }
    __syncthreads();  // everyone is done with stage s
    if (p.bulk && tid == 0 && i + p.stages < nt && is_bulk(t + p.stages)) {
      fence_proxy_async_smem();
      issue(t + p.stages, s);
    }
  }
  if (bail >= 0) {
    // Timeout recorded in *err; the host resets the ticket counter.  Copies already issued into
    // the ring (positions bail .. bail + stages - 1) may still be landing in shared memory:
    // wait for them, with the default bound, before the CTA exits.
    if (tid == 0)
      for (int j = bail; j < nt && j < bail + p.stages; j++)
        if (is_bulk(t_begin + j)) mbar_wait_bounded(&bars[j % p.stages], (uint32_t)((j / p.stages) & 1), nullptr);
    return;
  }

  // ---- CTA reduction ------------------------------------------------------------------------
  // The phases reduce into shared memory when (MN + NT) entries fit in the ring, otherwise
  // straight into this CTA's slot of the global partials (CTA-scope ordering by __syncthreads).
  const int MN = M * N;
  Acc* part = reinterpret_cast<Acc*>(p.partials);
  Acc* smem_red = reinterpret_cast<Acc*>(smem + SMEM_HEADER);
  const bool red_in_smem = gridDim.y == 1 && (size_t)(MN + NT) * sizeof(Acc) <= (size_t)p.smem_avail;
  Acc* red = red_in_smem ? smem_red : part + (size_t)blockIdx.x * MN;
  int nslots, slot;
  bool holder;
  if (32 % G == 0) {
#pragma unroll
    for (int x = 0; x < TM; x++)
#pragma unroll
      for (int y = 0; y < TN; y++)
        for (int o = G; o < 32; o <<= 1) acc[x][y] = O::add(acc[x][y], O::shfl_xor(acc[x][y], o));
    nslots = NT / 32;
    slot = tid / 32;
    holder = (tid % 32) < G;
  } else {
    nslots = RS;
    slot = rs;
    holder = active;
  }
  for (int sl = 0; sl < nslots; sl++) {
    if (holder && slot == sl) {
#pragma unroll
      for (int x = 0; x < TM; x++)
#pragma unroll
        for (int y = 0; y < TN; y++) {
          int m = m0 + x, n = n0 + y;
          if (m < M && n < N) red[n * M + m] = (sl == 0) ? acc[x][y] : O::add(red[n * M + m], acc[x][y]);
        }
    }
    __syncthreads();
  }
  if (red_in_smem)
    for (int e = tid; e < MN; e += NT) part[(size_t)blockIdx.x * MN + e] = red[e];
  __threadfence();
  __syncthreads();
  __shared__ int s_last;
  if (tid == 0) s_last = (atomicAdd(p.counter + blockIdx.y, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();

  // ---- last CTA: sum the CTA partials in CTA order, then the epilogue --------------------------
  const int nb = gridDim.x;
  if (gridDim.y == 1 && MN * 2 <= NT) {
    const int P = NT / MN;  // slices of the CTA range per entry
    const int e = tid % MN, j = tid / MN;
    Acc sum = O::zero();
    if (j < P) {
      int b0 = (int)((int64_t)nb * j / P), b1 = (int)((int64_t)nb * (j + 1) / P);
      for (int b = b0; b < b1; b++) sum = O::add(sum, ldcg(&part[(size_t)b * MN + e]));
    }
    Acc* red2 = smem_red + (red_in_smem ? MN : 0);  // P*MN <= NT entries
    if (j < P) red2[j * MN + e] = sum;
    __syncthreads();
    if (tid < MN) {
      Acc s = red2[tid];
      for (int q = 1; q < P; q++) s = O::add(s, red2[q * MN + tid]);
      int m = tid % M, n = tid / M;
      T* c = p.C + (int64_t)n * p.ldc + m;
      *c = O::finish(s, p.alpha, p.beta, p.beta_zero != 0, c);
    }
  } else {
    // entries owned by this group: cells [cbase, cbase + G), TM x TN each
    for (int q = tid; q < G * TM * TN; q += NT) {
      const int c = cbase + q / (TM * TN), x = (q % (TM * TN)) / TN, y = q % TN;
      const int m = (c % gm) * TM + x, n = (c / gm) * TN + y;
      if (m >= M || n >= N) continue;
      const int e = n * M + m;
      Acc s = O::zero();
      for (int b = 0; b < nb; b++) s = O::add(s, ldcg(&part[(size_t)b * MN + e]));
      T* cp = p.C + (int64_t)n * p.ldc + m;
      *cp = O::finish(s, p.alpha, p.beta, p.beta_zero != 0, cp);
    }
  }
  if (tid == 0) p.counter[blockIdx.y] = 0u;
}

}  // namespace skinny
