// split_tsmm.cu -- FP64 TSMM in split precision on tcgen05 tensor cores (no counterpart in the
// reference, whose FP64 TSMM kernels are CUDA-core DFMA loops, tsmm/fix3.cuh:4-39,
// tsmm/fix_fb.cuh:5-68).
//
// C(K x N) = alpha A(K x M) B(M x N) + beta C, B stored B[n*ldb+m], in place allowed (C == A).
//
// Scheme:
//   * alpha is folded into B once (FP64, one rounding per B element).  Column n of alpha*B gets a
//     shared exponent f_n; row r of A gets the exponent e_r of its largest element.  Every value
//     becomes a 62-bit fixed-point integer and 8 balanced base-256 digits (exact in BF16), as in
//     the split TSMTTSM (split.cu).
//   * The MMA contraction runs over (digit, column m).  A' (128 rows x 8*MP) holds A's digit planes
//     with the least significant first: plane p holds digit 8-p.  B' (N x 8*MP) holds B's planes
//     with the most significant first: plane q holds digit q+1.  For level L = i+j (2..9) the
//     product of the last (L-1) planes of A' with the first (L-1) planes of B' pairs exactly the
//     digits with i + j = L, so one MMA chain per level gives D_L(r, n) = sum_{i+j=L} sum_m a_i b_j.
//   * |D_L| <= 8 * MP * 2^14 <= 2^22 (MP <= 32): exact in the FP32 TMEM accumulator and exactly
//     convertible to int32 with a float add.
//   * Epilogue: V = sum_L D_L 2^(8(9-L)) as a 128-bit integer, rounded once to a double with
//     integer instructions, times 2^(e_r + f_n - 2112) in the exponent field; beta*C is one FMA.
//     Levels >= 10 are dropped (weight below 2^-56 of the leading level).
//   * Tiles of 128 rows stream through a ring of FP64 tiles (1-D TMA bulk copies); the MMAs of tile
//     t overlap the epilogue of tile t-1 (double-buffered TMEM accumulators).
// Complex FP64 (interleaved) runs as the real product of doubled width: A (K x 2M), B' (2M x 2N)
// with B'[2n][2m] = br, B'[2n][2m+1] = -bi, B'[2n+1][2m] = bi, B'[2n+1][2m+1] = br, C (K x 2N).
// Inputs must be finite.
#include <cuda_bf16.h>

#include <cstring>

#include "api_internal.h"

namespace skinny {
namespace stsmm {

constexpr int ROWS = 128;
constexpr int THREADS = 256;
constexpr int DIGITS = 8;
constexpr int HDR = 4096;      // barriers, TMEM slot, row/column exponents
constexpr int BAL = 8192;      // alpha*B staging (<= 32 x 32 doubles)

struct Args {
  const double* A;
  const double* B;  // real: B[n*ldb+m]; complex: the complex B (interleaved)
  double* C;
  int64_t K, lda, ldb, ldc;  // in doubles (complex: already doubled)
  int M, N;                  // real widths (complex: 2M, 2N)
  int MP, NM;                // padded contraction width (16 or 32), MMA N (16 or 32)
  int cplx;                  // B is complex (alpha, beta complex)
  double alpha[2], beta[2];
  int beta_zero, inplace, bulk, stages;
  int64_t ntiles;
  uint32_t tile_bytes;  // FP64 stage bytes
  int64_t lda_s;        // row stride of the FP64 stage tile
  int wload;            // columns staged by plain loads (in place: max(M, N), beta*C reads them)
  uint32_t abuf;        // bytes of one A' buffer
  int nabuf;            // A' buffers (1 or 2)
  int tmem_cols;
  int* err;
};

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((128 >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ uint32_t exp_field(double x) {
  uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  uint32_t ef = (hi >> 20) & 0x7FF;
  bool nz = ((hi & 0x7FFFFFFFu) | lo) != 0;
  return nz ? (ef ? ef : 1u) : 0u;
}

// 8 balanced digits of x relative to exponent field E (most significant first), as exact floats
__device__ __forceinline__ void digits_of(double x, uint32_t E, float (&d)[DIGITS], bool& neg) {
  uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  uint32_t ef = (hi >> 20) & 0x7FF;
  neg = (hi >> 31) != 0;
  uint32_t eff = ef ? ef : 1u;
  uint64_t mant = ((uint64_t)((hi & 0xFFFFFu) | (ef ? 0x100000u : 0u)) << 32) | lo;
  uint32_t sh = E - eff;
  uint64_t F = sh < 64 ? ((mant << 9) >> sh) : 0ull;
  uint64_t G = F + 0x8080808080808080ull;
  uint32_t gh = (uint32_t)(G >> 32), gl = (uint32_t)G;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    d[i] = __uint_as_float(0x4B000000u | ((gh >> (8 * (3 - i))) & 0xFF)) - 8388736.0f;
    d[4 + i] = __uint_as_float(0x4B000000u | ((gl >> (8 * (3 - i))) & 0xFF)) - 8388736.0f;
  }
}

__device__ __forceinline__ uint32_t pack2(float a, float b, bool na, bool nb) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  uint32_t u = *reinterpret_cast<uint32_t*>(&h);
  return u ^ ((na ? 0x8000u : 0u) | (nb ? 0x80000000u : 0u));
}

// K-major no-swizzle operand: element (row, k) of a tile whose k-octets are lbo bytes apart
__device__ __forceinline__ uint32_t kmaj(int row, int koct, uint32_t lbo) {
  return (uint32_t)koct * lbo + (uint32_t)(row >> 3) * 128u + (uint32_t)(row & 7) * 16u;
}

// round the signed 128-bit integer (hi:lo) to the nearest double and scale by 2^E (E applied to
// the exponent field; results are assumed to stay in the normal range)
__device__ __forceinline__ double i128_to_double(long long hi, unsigned long long lo, int E) {
  const bool neg = hi < 0;
  unsigned long long h = (unsigned long long)hi, l = lo;
  if (neg) {  // two's complement negate
    l = ~l + 1ull;
    h = ~h + (l == 0ull ? 1ull : 0ull);
  }
  if ((h | l) == 0ull) return 0.0;
  int P;  // position of the leading one
  unsigned long long top;  // 64 bits starting at the leading one
  bool sticky;
  if (h) {
    const int z = __clzll((long long)h);
    P = 127 - z;
    top = z ? ((h << z) | (l >> (64 - z))) : h;
    sticky = z ? ((l << z) != 0ull) : (l != 0ull);
  } else {
    const int z = __clzll((long long)l);
    P = 63 - z;
    top = l << z;
    sticky = false;
  }
  unsigned long long mant = top >> 11;  // 53 bits
  const unsigned long long rem = top & 0x7FFull;
  sticky = sticky || ((rem & 0x3FFull) != 0ull);
  const bool half = (rem & 0x400ull) != 0ull;
  if (half && (sticky || (mant & 1ull))) mant++;
  int ex = P + E;
  if (mant >> 53) {
    mant >>= 1;
    ex++;
  }
  const long long bits = ((long long)(ex + 1023) << 52) | (long long)(mant & 0xFFFFFFFFFFFFFull);
  const double v = __longlong_as_double(bits);
  return neg ? -v : v;
}

__global__ void __launch_bounds__(THREADS, 1) split_tsmm_kernel(const Args p) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bar_tma = reinterpret_cast<uint64_t*>(smem);        // [4]
  uint64_t* bar_mma = reinterpret_cast<uint64_t*>(smem + 32);   // [2]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 64);
  int* erow = reinterpret_cast<int*>(smem + 128);               // [2][2][ROWS]: tile parity, half
  int* fcol = reinterpret_cast<int*>(smem + 128 + 4 * ROWS * 4);  // [32]
  const int M = p.M, N = p.N, MP = p.MP, NM = p.NM;
  const uint32_t lbo_a = ROWS * 16, lbo_b = (uint32_t)NM * 16;
  unsigned char* bdig = smem + HDR + BAL;                         // B' (NM x 8*MP), 1024-aligned
  const uint32_t bdig_bytes = (uint32_t)(8 * MP / 8) * lbo_b;
  unsigned char* adig = bdig + ((bdig_bytes + 1023) & ~1023u);   // A' buffers
  unsigned char* ring = adig + (size_t)p.nabuf * p.abuf;
  double* bal = reinterpret_cast<double*>(smem + HDR);           // alpha*B as [m][n]
  auto tile = [&](int s) { return reinterpret_cast<double*>(ring + (size_t)s * p.tile_bytes); };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t t_begin = p.ntiles * blockIdx.x / gridDim.x;
  const int64_t t_end = p.ntiles * (blockIdx.x + 1) / gridDim.x;
  const int nt = (int)(t_end - t_begin);
  auto is_bulk = [&](int64_t t) { return p.bulk && (t + 1) * (int64_t)ROWS < p.K; };
  auto issue = [&](int64_t t, int s) {
    const uint32_t b = (uint32_t)(ROWS * p.lda * 8);
    mbar_arrive_expect_tx(&bar_tma[s], b);
    bulk_g2s(tile(s), p.A + t * ROWS * p.lda, b, &bar_tma[s]);
  };

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(p.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < p.stages; s++) mbar_init(&bar_tma[s], 1);
    mbar_init(&bar_mma[0], 1);
    mbar_init(&bar_mma[1], 1);
    fence_mbar_init();
  }
  // ---- alpha * B (FP64) as bal[m][n], column exponents, B' digits -----------------------------
  // B' row n: plane q (digit q+1) at k = q*MP + m; entries for m >= M or n >= N are zero
  for (int e = tid; e < MP * NM; e += THREADS) {
    const int m = e / NM, n = e % NM;
    double v = 0.0;
    if (m < M && n < N) {
      if (!p.cplx) {
        v = p.B[(int64_t)n * p.ldb + m] * p.alpha[0];
      } else {  // real view of complex B: (2n + s, 2m + t)
        const int nc = n >> 1, mc = m >> 1;
        const double br = p.B[2 * ((int64_t)nc * p.ldb + mc)], bi = p.B[2 * ((int64_t)nc * p.ldb + mc) + 1];
        const double ar = br * p.alpha[0] - bi * p.alpha[1], ai = br * p.alpha[1] + bi * p.alpha[0];
        v = ((n & 1) == 0) ? ((m & 1) == 0 ? ar : -ai) : ((m & 1) == 0 ? ai : ar);
      }
    }
    bal[m * NM + n] = v;
  }
  if (tid < 32) fcol[tid] = 0;
  __syncthreads();
  if (tid < NM) {
    uint32_t f = 0;
    for (int m = 0; m < MP; m++) f = max(f, exp_field(bal[m * NM + tid]));
    fcol[tid] = (int)f;
  }
  __syncthreads();
  for (int u = tid; u < NM * (MP / 8); u += THREADS) {  // unit: (n, m-octet)
    const int n = u % NM, mo = u / NM;
    float d[8][DIGITS];
    bool ng[8];
#pragma unroll
    for (int q2 = 0; q2 < 8; q2++) digits_of(bal[(mo * 8 + q2) * NM + n], (uint32_t)fcol[n], d[q2], ng[q2]);
#pragma unroll
    for (int j = 0; j < DIGITS; j++) {
      uint4 w = make_uint4(pack2(d[0][j], d[1][j], ng[0], ng[1]), pack2(d[2][j], d[3][j], ng[2], ng[3]),
                           pack2(d[4][j], d[5][j], ng[4], ng[5]), pack2(d[6][j], d[7][j], ng[6], ng[7]));
      *reinterpret_cast<uint4*>(bdig + kmaj(n, (j * MP + mo * 8) / 8, lbo_b)) = w;
    }
  }
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *tslot;
  if (p.bulk && tid == 0)
    for (int i = 0; i < nt && i < p.stages; i++)
      if (is_bulk(t_begin + i)) issue(t_begin + i, i);

  const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(NM >> 3) << 17) | ((128u >> 4) << 24);
  const int row = tid & (ROWS - 1), half = tid >> 7;  // slicing: 2 threads per row
  int uses[2] = {0, 0};
  bool bail = false;

  // epilogue of local tile `it` (TMEM buffer it & 1)
  auto epilogue = [&](int it) {
    const int64_t t = t_begin + it;
    const int64_t r0 = t * ROWS;
    const int rows = (int)((p.K - r0) < ROWS ? (p.K - r0) : ROWS);
    const int b = it & 1;
    const int q = warp & 3;
    const int r = 32 * q + lane;
    const int* er = erow + (b * 2) * ROWS;  // both halves hold the row maximum
    const uint32_t tbase = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * 8 * NM);
    const double* T = tile(it % p.stages);
    // n range of this warp: warps 0-3 take the low half of the columns, 4-7 the high half
    const int nh = min(N, (((N + 1) / 2) + 1) & ~1);  // even split keeps complex (re, im) pairs together
    const int n0 = (warp < 4) ? 0 : nh, n1 = (warp < 4) ? nh : N;
    for (int c0 = (n0 & ~7); c0 < n1; c0 += 8) {
      uint32_t raw[8][8];
#pragma unroll
      for (int L = 0; L < 8; L++) tmem_ld8(tbase + (uint32_t)(L * NM + c0), raw[L]);
      tmem_wait();
      if (r < rows) {
        const int e = er[r];
        double* crow = p.C + (r0 + r) * p.ldc;
        // old C values of the chunk are read before any of them is overwritten
        double cold[8];
#pragma unroll
        for (int x = 0; x < 8; x++) {
          const int n = c0 + x;
          cold[x] = (!p.beta_zero && n >= n0 && n < n1) ? (p.inplace ? T[r * p.lda_s + n] : crow[n]) : 0.0;
        }
        double out[8];
#pragma unroll
        for (int x = 0; x < 8; x++) {
          const int n = c0 + x;
          out[x] = 0.0;
          if (n < n0 || n >= n1) continue;
          long long dl[8];
#pragma unroll
          for (int L = 0; L < 8; L++)
            dl[L] = (long long)(__float_as_int(__uint_as_float(raw[L][x]) + 12582912.0f) - 0x4B400000);
          const long long H = (dl[0] << 24) + (dl[1] << 16) + (dl[2] << 8) + dl[3];  // levels 2..5
          const long long Lo = (dl[4] << 24) + (dl[5] << 16) + (dl[6] << 8) + dl[7]; // levels 6..9
          // V = H * 2^32 + Lo as 128 bits
          const long long Hh = H >> 32;
          const unsigned long long Hl = (unsigned long long)H & 0xFFFFFFFFull;
          const unsigned long long lo0 = Hl << 32;
          const unsigned long long lo1 = lo0 + (unsigned long long)Lo;
          const long long hi1 = Hh + (lo1 < lo0 ? 1 : 0) + (Lo < 0 ? -1 : 0);
          double v = i128_to_double(hi1, lo1, e + fcol[n] - 2112);
          if (!p.beta_zero) {
            if (!p.cplx) {
              v = fma(p.beta[0], cold[x], v);
            } else {  // (re, im) = (cold[x & ~1], cold[x | 1]); c0 is a multiple of 8
              const double cr = cold[x & ~1], ci = cold[x | 1];
              v = (n & 1) ? fma(p.beta[0], ci, fma(p.beta[1], cr, v)) : fma(p.beta[0], cr, fma(-p.beta[1], ci, v));
            }
          }
          out[x] = v;
        }
#pragma unroll
        for (int x = 0; x < 8; x++) {
          const int n = c0 + x;
          if (n >= n0 && n < n1) crow[n] = out[x];
        }
      }
    }
  };

  for (int it = 0; it < nt && !bail; it++) {
    const int64_t t = t_begin + it;
    const int s = it % p.stages;
    const int64_t r0 = t * ROWS;
    const int rows = (int)((p.K - r0) < ROWS ? (p.K - r0) : ROWS);
    double* T = tile(s);
    if (is_bulk(t)) {
      bool ok = mbar_wait_bounded(&bar_tma[s], (uint32_t)((it / p.stages) & 1), p.err);
      if (__syncthreads_or(!ok)) {
        bail = true;
        break;
      }
    } else {
      const int W = p.wload;
      for (int e = tid; e < rows * W; e += THREADS) {
        const int rr = e / W, c = e - rr * W;
        T[rr * p.lda_s + c] = p.A[(r0 + rr) * p.lda + c];
      }
      __syncthreads();
    }
    // row exponents (two threads per row: each half of the columns)
    const int mh = MP / 2, mlo = half * mh;
    uint32_t emax = 0;
    if (row < rows)
      for (int m = mlo; m < mlo + mh && m < M; m++) emax = max(emax, exp_field(T[row * p.lda_s + m]));
    int* er = erow + ((it & 1) * 2) * ROWS;
    er[half * ROWS + row] = (int)emax;
    // A' buffer free? (the MMAs of tile it - nabuf have completed)
    const int ab = it % p.nabuf;
    __syncthreads();
    const int e_row = max(er[row], er[ROWS + row]);
    if (p.nabuf == 1 && it > 0) {
      const int bp = (it - 1) & 1;
      bool ok = mbar_wait_bounded(&bar_mma[bp], (uint32_t)((uses[bp] - 1) & 1), p.err);
      if (__syncthreads_or(!ok)) {
        bail = true;
        break;
      }
    } else if (p.nabuf == 2 && it > 1) {
      const int bp = it & 1;  // tile it-2 used TMEM/bar parity it & 1 as well
      bool ok = mbar_wait_bounded(&bar_mma[bp], (uint32_t)((uses[bp] - 1) & 1), p.err);
      if (__syncthreads_or(!ok)) {
        bail = true;
        break;
      }
    }
    // slice: thread (row, half) writes, for each octet of its half of the columns, the 8 digit
    // planes p = 0..7 (digit 8 - p) at k = p * MP + m
    unsigned char* A_ = adig + (size_t)ab * p.abuf;
    for (int mo = mlo / 8; mo < (mlo + mh) / 8; mo++) {
      float d[8][DIGITS];
      bool ng[8];
#pragma unroll
      for (int q2 = 0; q2 < 8; q2++) {
        const int m = mo * 8 + q2;
        const double x = (row < rows && m < M) ? T[row * p.lda_s + m] : 0.0;
        digits_of(x, (uint32_t)e_row, d[q2], ng[q2]);
      }
#pragma unroll
      for (int pl = 0; pl < DIGITS; pl++) {
        const int i = 7 - pl;  // digit index (0-based) stored in plane pl
        uint4 w = make_uint4(pack2(d[0][i], d[1][i], ng[0], ng[1]), pack2(d[2][i], d[3][i], ng[2], ng[3]),
                             pack2(d[4][i], d[5][i], ng[4], ng[5]), pack2(d[6][i], d[7][i], ng[6], ng[7]));
        *reinterpret_cast<uint4*>(A_ + kmaj(row, (pl * MP + mo * 8) / 8, lbo_a)) = w;
      }
    }
    if (tid < ROWS) er[tid] = e_row;  // the epilogue of this tile reads er[r]
    fence_proxy_async_smem();
    tc_before();
    __syncthreads();
    if (tid == 0) {
      tc_after();
      const int b = it & 1;
      const uint32_t a0 = smem_u32(A_), b0 = smem_u32(bdig);
      const uint32_t dcol = tmem + (uint32_t)(b * 8 * NM);
      for (int L = 2; L <= 9; L++) {
        const int kq = (L - 1) * MP / 16;    // K-steps of 16
        const int ka = (9 - L) * MP / 8;     // first k-octet of A' for this level
        for (int ks = 0; ks < kq; ks++)
          mma_bf16(dcol + (uint32_t)((L - 2) * NM), make_desc(a0 + (uint32_t)(ka + 2 * ks) * lbo_a, lbo_a),
                   make_desc(b0 + (uint32_t)(2 * ks) * lbo_b, lbo_b), idesc, ks > 0 ? 1u : 0u);
      }
      mma_commit(&bar_mma[b]);
    }
    uses[it & 1]++;
    // epilogue of the previous tile overlaps this tile's MMAs
    if (it > 0) {
      const int bp = (it - 1) & 1;
      bool ok = mbar_wait_bounded(&bar_mma[bp], (uint32_t)((uses[bp] - 1) & 1), p.err);
      if (__syncthreads_or(!ok)) {
        bail = true;
        break;
      }
      tc_after();
      epilogue(it - 1);
      tc_before();
      __syncthreads();
      // FP64 stage of tile it-1 is free now (its epilogue may have read it in place)
      if (tid == 0 && p.bulk) {
        const int sp = (it - 1) % p.stages;
        const int64_t tn = t - 1 + p.stages;
        if (it - 1 + p.stages < nt && is_bulk(tn)) {
          fence_proxy_async_smem();
          issue(tn, sp);
        }
      }
    }
  }
  if (!bail && nt > 0) {
    const int bl = (nt - 1) & 1;
    bool ok = mbar_wait_bounded(&bar_mma[bl], (uint32_t)((uses[bl] - 1) & 1), p.err);
    if (__syncthreads_or(!ok)) {
      bail = true;
    } else {
      tc_after();
      epilogue(nt - 1);
    }
  }
  if (bail)
    for (int bb = 0; bb < 2; bb++)
      if (uses[bb] > 0) mbar_wait_bounded(&bar_mma[bb], (uint32_t)((uses[bb] - 1) & 1), nullptr);
  tc_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.tmem_cols));
}

}  // namespace stsmm

skinny_status split_tsmm(skinny_handle h, bool cplx, int64_t M, int64_t N, int64_t K, const double* A,
                         int64_t lda, const void* alpha, const double* B, int64_t ldb, const void* beta, double* C,
                         int64_t ldc, cudaStream_t st, bool autoselect) {
  using namespace stsmm;
  const int64_t Mr = cplx ? 2 * M : M, Nr = cplx ? 2 * N : N;
  if (Mr > 32 || Nr > 32) {
    set_error("split precision TSMM: real widths M, N <= 32 in this build");
    return SKINNY_UNSUPPORTED;
  }
  // auto selection (measured on GB300): split wins from real widths Mr * Nr >= 512 on (FP64 32x32,
  // complex 16x16); below that the CUDA-core kernels are as fast.  The autotuner can override.
  if (autoselect && (K < 8192 || Mr * Nr < 512)) {
    set_error("split precision TSMM: not selected automatically for this shape");
    return SKINNY_UNSUPPORTED;
  }
  Args a;
  a.A = A;
  a.B = B;
  a.C = C;
  a.K = K;
  a.lda = cplx ? 2 * lda : lda;
  a.ldb = ldb;
  a.ldc = cplx ? 2 * ldc : ldc;
  a.M = (int)Mr;
  a.N = (int)Nr;
  a.MP = Mr <= 16 ? 16 : 32;
  a.NM = Nr <= 16 ? 16 : 32;
  a.cplx = cplx;
  std::memset(a.alpha, 0, sizeof a.alpha);
  std::memset(a.beta, 0, sizeof a.beta);
  std::memcpy(a.alpha, alpha, cplx ? 16 : 8);
  std::memcpy(a.beta, beta, cplx ? 16 : 8);
  a.beta_zero = a.beta[0] == 0.0 && a.beta[1] == 0.0;
  a.inplace = (const void*)A == (const void*)C;
  const bool aligned = (uintptr_t)A % 16 == 0;
  const bool dense = a.lda <= 2 * Mr + 16;
  a.bulk = aligned && dense && K > ROWS;
  a.wload = (int)(a.inplace ? std::max(Mr, Nr) : Mr);
  a.lda_s = a.bulk ? a.lda : a.wload;
  a.tile_bytes = (uint32_t)round_up(ROWS * a.lda_s * 8, 1024);
  a.abuf = (uint32_t)(ROWS * 8 * a.MP * 2);  // 128 rows x 8 planes x MP x bf16
  const uint32_t bdig = (uint32_t)round_up((int64_t)8 * a.MP * a.NM * 2, 1024);
  const int64_t fixed = HDR + BAL + bdig;
  a.nabuf = 2;
  int stages = (int)std::min<int64_t>(4, (h->dev.smem_optin - fixed - 2 * (int64_t)a.abuf) / a.tile_bytes);
  if (stages < 3) {
    a.nabuf = 1;
    stages = (int)std::min<int64_t>(4, (h->dev.smem_optin - fixed - (int64_t)a.abuf) / a.tile_bytes);
  }
  if (stages < 2 || (a.inplace && stages < 3)) {
    set_error("split precision TSMM: tiles do not fit in shared memory");
    return SKINNY_UNSUPPORTED;
  }
  a.stages = stages;
  a.ntiles = (K + ROWS - 1) / ROWS;
  a.tmem_cols = 2 * 8 * a.NM <= 256 ? 256 : 512;
  a.err = h->err;
  const int smem = (int)(fixed + (int64_t)a.nabuf * a.abuf + (int64_t)stages * a.tile_bytes);
  int64_t grid = std::min<int64_t>(h->dev.sms, a.ntiles);
  if (grid < 1) grid = 1;
  static std::atomic<int> attr{0};
  ensure_smem_attr(split_tsmm_kernel, smem, attr);
  split_tsmm_kernel<<<(int)grid, THREADS, smem, st>>>(a);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("split tsmm launch: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  return SKINNY_OK;
}

}  // namespace skinny
