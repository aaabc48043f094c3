// split_tsmm.cu -- FP64 TSMM in split precision on tcgen05 tensor cores (no counterpart in the
// reference, whose FP64 TSMM kernels are CUDA-core DFMA loops, tsmm/fix3.cuh:4-39,
// tsmm/fix_fb.cuh:5-68).
//
// C(K x N) = alpha A(K x M) B(M x N) + beta C, B stored B[n*ldb+m], in place allowed (C == A).
//
// Scheme:
//   * alpha is folded into B once (FP64, one rounding per B element).  Column n of alpha*B gets a
//     shared exponent f_n; row r of A gets the exponent e_r of its largest element.  Every value
//     becomes a 62-bit fixed-point integer and 8 balanced base-256 digits (exact in FP16), as in
//     the split TSMTTSM (split.cu); A's digits are formed with byte permutes and one HFMA2 per
//     digit pair (digit_pairs).
//   * The MMA contraction runs over (digit, column m).  A' (128 rows x 8*MP) holds A's digit planes
//     with the least significant first: plane p holds digit 8-p.  B' (N x 8*MP) holds B's planes
//     with the most significant first: plane q holds digit q+1.  For level L = i+j (2..9) the
//     product of the last (L-1) planes of A' with the first (L-1) planes of B' pairs exactly the
//     digits with i + j = L, so one MMA chain per level gives D_L(r, n) = sum_{i+j=L} sum_m a_i b_j.
//   * |D_L| <= 8 * MP * 2^14 <= 2^23: exact in the FP32 TMEM accumulator.
//   * Epilogue: V = sum_L D_L 2^(8(9-L)) (< 2^80) is formed in integers (level pairs in 32 bits),
//     its top 61+ bits (from its own leading bit; the rest lies below 2^-61 of |V|) are rounded to
//     a double with integer instructions and scaled by 2^(e_r + f_n - 2112) in the exponent field;
//     beta*C is one FMA (the only FP64-pipe operation per output).
//     Levels >= 10 are dropped (weight below 2^-56 of the leading level).
//   * Tiles of 128 rows: two threads per row (contraction width 16; four above, with 16 warps per
//     CTA) read the row's FP64 values straight from global memory into registers; the next
//     tile's values are loaded right after the current one is sliced, behind the epilogue; the
//     MMAs of tile t overlap the epilogue of tile t-1 where two TMEM accumulators fit (N <= 32).
//     Four threads issue the level chains (levels 2+w and 9-w from warp w: 9*MP/16 MMAs each), so
//     no single warp serialises the whole tile's MMAs.  The epilogue reads the old C values of a
//     chunk before the TMEM loads of the chunk before it (16-byte pieces where rows are aligned),
//     so that global and TMEM latencies overlap.
//   * |D_L| <= 2^22 for contraction widths <= 32 (converted with a float add), <= 2^23 for 64
//     (converted with integer instructions from the FP32 bit pattern); both exact.
//   * In place with M == N, beta is folded into the diagonal of alpha*B before slicing
//     (C = A (alpha B + beta I)), so the epilogue neither reads C nor runs the beta FMA.
// Complex FP64 (interleaved) runs as the real product of doubled width: A (K x 2M), B' (2M x 2N)
// with B'[2n][2m] = br, B'[2n][2m+1] = -bi, B'[2n+1][2m] = bi, B'[2n+1][2m+1] = br, C (K x 2N).
// Inputs must be finite.
#include <cuda_fp16.h>

#include <cstring>

#include "api_internal.h"
#include "digits.cuh"

namespace skinny {
namespace stsmm {

constexpr int ROWS = 128;
// threads: 256 when two CTAs share an SM (contraction width 16, accumulators of <= 256 columns),
// otherwise 512 (one CTA of 16 warps per SM); 128 registers either way.  Rows are sliced by up to
// four threads each (8 columns at least per thread); the epilogue splits the columns over NT/128
// warp groups -- enough warps to cover its TMEM and global latencies.
constexpr int DIGITS = 8;
constexpr int HDR = 8192;      // barriers, TMEM slot, row/column exponents

struct Args {
  const double* A;
  const double* B;  // real: B[n*ldb+m]; complex: the complex B (interleaved)
  double* C;
  int64_t K, lda, ldb, ldc;  // in doubles (complex: lda, ldc already doubled; ldb in complex elements)
  int M, N;                  // real widths (complex: 2M, 2N)
  int NM;                    // MMA N: 16, 32 or 64
  int cplx;                  // B is complex (alpha, beta complex)
  double alpha[2], beta[2];
  int beta_zero, inplace, vec;  // vec: rows of A may be read as 16-byte pairs
  int fold;                     // beta folded into B's diagonal (in place, M == N); beta_zero then set
  int vecc;                     // rows of C may be read and written as 16-byte pairs
  int64_t ntiles;
  uint32_t abuf;  // bytes of one A' buffer
  int nabuf;      // A' buffers (1 or 2)
  int ntbuf;      // TMEM accumulator buffers (1 or 2)
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
__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
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
  uint32_t gh, gl;
  g_words(x, E, gh, gl, neg);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    d[i] = __uint_as_float(0x4B000000u | ((gh >> (8 * (3 - i))) & 0xFF)) - 8388736.0f;
    d[4 + i] = __uint_as_float(0x4B000000u | ((gl >> (8 * (3 - i))) & 0xFF)) - 8388736.0f;
  }
}

// two FP16 digits (a in the low half), signs applied
__device__ __forceinline__ uint32_t pack2(float a, float b, bool na, bool nb) {
  __half2 h = __floats2half2_rn(a, b);
  uint32_t u = *reinterpret_cast<uint32_t*>(&h);
  return u ^ ((na ? 0x8000u : 0u) | (nb ? 0x80000000u : 0u));
}

// K-major no-swizzle operand: element (row, k) of a tile whose k-octets are lbo bytes apart
__device__ __forceinline__ uint32_t kmaj(int row, int koct, uint32_t lbo) {
  return (uint32_t)koct * lbo + (uint32_t)(row >> 3) * 128u + (uint32_t)(row & 7) * 16u;
}

// value of (alpha * B + fold * I) at (m, n) in the real view, 0 outside M x N; fold is beta for
// the in-place product with M == N (C = A (alpha B + beta I)), else 0
__device__ __forceinline__ double alpha_b(const Args& p, int m, int n) {
  if (m >= p.M || n >= p.N) return 0.0;
  if (!p.cplx) {
    const double v = p.B[(int64_t)n * p.ldb + m] * p.alpha[0];
    return (p.fold && m == n) ? v + p.beta[0] : v;
  }
  const int nc = n >> 1, mc = m >> 1;
  const double br = p.B[2 * ((int64_t)nc * p.ldb + mc)], bi = p.B[2 * ((int64_t)nc * p.ldb + mc) + 1];
  double ar = br * p.alpha[0] - bi * p.alpha[1], ai = br * p.alpha[1] + bi * p.alpha[0];
  if (p.fold && mc == nc) {
    ar += p.beta[0];
    ai += p.beta[1];
  }
  return ((n & 1) == 0) ? ((m & 1) == 0 ? ar : -ai) : ((m & 1) == 0 ? ai : ar);
}

// A row values of this thread's half of the columns (MP/2 values) for tile row r0 + row
template <int HALF>
__device__ __forceinline__ void load_row(const Args& p, int64_t r0, int row, int rows, int m0, double (&v)[HALF]) {
  const bool ok = row < rows;
  const double* a = p.A + (r0 + row) * p.lda + m0;
  if (ok && p.vec && m0 + HALF <= p.M) {
#pragma unroll
    for (int j = 0; j < HALF; j += 2) {
      double2 x = p.inplace ? *reinterpret_cast<const double2*>(a + j) : __ldg(reinterpret_cast<const double2*>(a + j));
      v[j] = x.x;
      v[j + 1] = x.y;
    }
  } else {
#pragma unroll
    for (int j = 0; j < HALF; j++) v[j] = (ok && m0 + j < p.M) ? a[j] : 0.0;
  }
}

// x * 2^E for a signed 64-bit integer x, rounded to 53 bits (ties away from zero); |x| < 2^63,
// 0 for x == 0.  Branch-free: for x == 0 the normalising shift is masked to 0 and the final select
// returns 0.
__device__ __forceinline__ double i64_to_double(long long x, int E) {
  const unsigned long long sgn = (unsigned long long)x & 0x8000000000000000ull;
  unsigned long long m = (unsigned long long)(x < 0 ? -x : x);
  const int z = __clzll((long long)m);  // >= 1 for x != 0
  m <<= (z & 63);                       // leading one at bit 63
  unsigned long long mant = (m + 0x400ull) >> 11;  // round on bit 10; may carry to 2^53
  int ex = 63 - z + E;
  const unsigned long long carry = mant >> 53;
  mant >>= carry;
  ex += (int)carry;
  const double r =
      __longlong_as_double((long long)(sgn | ((unsigned long long)(ex + 1023) << 52) | (mant & 0xFFFFFFFFFFFFFull)));
  return x ? r : 0.0;
}

// The integer value of an FP32 holding an exact integer with |f| < 2^24, with integer instructions
// only (a float-to-int conversion instruction shares GB300's narrow FP64 pipe, the unit the beta
// FMA already needs): the mantissa with its implicit bit, shifted right by 150 - exponent (a
// funnel shift that clamps at 32, so 0.0 gives 0), then the sign.
__device__ __forceinline__ int f32_int_exact(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t mag = __funnelshift_rc((u & 0x7FFFFFu) | 0x800000u, 0u, 150u - ((u >> 23) & 0xFFu));
  const int s = (int)u >> 31;  // 0 or -1
  return ((int)mag ^ s) - s;
}

// The double of column x of a chunk: V = sum_L D_L 2^(8(9-L)) from the eight FP32 level sums in
// raw[L][x] (exact integers), times 2^E.
template <int MP>
__device__ __forceinline__ double level_value(const uint32_t (&raw)[8][8], int x, int E) {
  int dl[8];
#pragma unroll
  for (int L = 0; L < 8; L++) {
    const float f = __uint_as_float(raw[L][x]);
    // |D_L| <= (L-1) * MP * 2^14: up to 2^22 the magic add is exact (levels 2..5 at MP = 64)
    dl[L] = (MP <= 32 || L < 4) ? __float_as_int(f + 12582912.0f) - 0x4B400000 : f32_int_exact(f);
  }
  // level pairs in 32 bits: |D_L * 256 + D_{L+1}| < 2^31 for every pair (the largest, D_8 * 256 +
  // D_9 at MP = 64, is below 1.9e9)
  const int P1 = dl[0] * 256 + dl[1], P2 = dl[2] * 256 + dl[3];
  const int P3 = dl[4] * 256 + dl[5], P4 = dl[6] * 256 + dl[7];
  // H = levels 2..5, Lo = levels 6..9 (each |.| < 2^48), V = H * 2^32 + Lo < 2^80.
  const long long H = ((long long)P1 << 16) + P2;
  const long long Lo = ((long long)P3 << 16) + P4;
  // the top bits of V from its own leading bit: shift H up by k = clz(|H|) - 2, so that
  // |H << k| < 2^62 and adding the |Lo| part (< 2^48) cannot pass 2^63 (k = 32, also for H = 0:
  // V fits in 64 bits and is kept whole); at least 61 bits are kept, the bits of Lo dropped lie
  // below 2^-61 of |V|.  They are rounded to a double with integer instructions (a conversion
  // instruction from 64-bit integers runs on the FP64 pipe, the scarce unit here)
  const long long aH = H < 0 ? -H : H;
  const int k = min(32, __clzll(aH) - 2);
  const long long top = (H << k) + (Lo >> (32 - k));
  return i64_to_double(top, E - k);
}

// contraction width 16 (TMEM <= 256 columns, shared memory < 114 KB): two CTAs per SM, so that one
// CTA's barriers overlap the other's work
template <int MP, int NT>
__global__ void __launch_bounds__(NT, NT == 256 ? 2 : 1) split_tsmm_kernel(const Args p) {
  constexpr int TPR = NT / ROWS;                         // column parts of the epilogue
  constexpr int TPS = MP / 8 < TPR ? MP / 8 : TPR;       // threads slicing a row
  constexpr int PART = MP / TPS;                         // columns sliced per thread
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bar_mma = reinterpret_cast<uint64_t*>(smem + 32);   // [2]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 64);
  int* erow = reinterpret_cast<int*>(smem + 128);               // [2 parity][TPR parts][ROWS]
  int* fcol = reinterpret_cast<int*>(smem + 128 + 2 * TPR * ROWS * 4);  // [64]
  const int M = p.M, N = p.N, NM = p.NM;
  const uint32_t lbo_a = ROWS * 16, lbo_b = (uint32_t)NM * 16;
  unsigned char* bdig = smem + HDR;                               // B' (NM x 8*MP), 1024-aligned
  const uint32_t bdig_bytes = (uint32_t)(8 * MP / 8) * lbo_b;
  unsigned char* adig = bdig + ((bdig_bytes + 1023) & ~1023u);   // A' buffers

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t t_begin = p.ntiles * blockIdx.x / gridDim.x;
  const int64_t t_end = p.ntiles * (blockIdx.x + 1) / gridDim.x;
  const int nt = (int)(t_end - t_begin);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(p.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {  // four issuing threads commit to each tile's barrier
    mbar_init(&bar_mma[0], 4);
    mbar_init(&bar_mma[1], 4);
    fence_mbar_init();
  }
  // ---- B' = digits of alpha * B: column exponents, then (n, m-octet) units -------------------
  if (tid < NM) {
    uint32_t f = 0;
    for (int m = 0; m < M; m++) f = max(f, exp_field(alpha_b(p, m, tid)));
    fcol[tid] = (int)f;
  }
  __syncthreads();
  for (int u = tid; u < NM * (MP / 8); u += NT) {
    const int n = u % NM, mo = u / NM;
    float d[8][DIGITS];
    bool ng[8];
#pragma unroll
    for (int q2 = 0; q2 < 8; q2++) digits_of(alpha_b(p, mo * 8 + q2, n), (uint32_t)fcol[n], d[q2], ng[q2]);
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

  // kind::f16 with FP16 A and B (a/b format 0), FP32 accumulators, N = NM, M = 128
  const uint32_t idesc = (1u << 4) | ((uint32_t)(NM >> 3) << 17) | ((128u >> 4) << 24);
  const int row = tid & (ROWS - 1), part = tid >> 7;
  const bool slicer = part < TPS;
  const int m0 = (slicer ? part : 0) * PART;
  int uses[2] = {0, 0};
  bool bail = false;

  auto epilogue = [&](int it) {
    const int64_t t = t_begin + it;
    const int64_t r0 = t * ROWS;
    const int rows = (int)((p.K - r0) < ROWS ? (p.K - r0) : ROWS);
    const int q = warp & 3;
    const int r = 32 * q + lane;
    const int* er = erow + ((it & 1) * TPR) * ROWS;
    const uint32_t tbase = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)((it % p.ntbuf) * 8 * NM);
    // TPR column parts of even width (complex (re, im) pairs stay together), one per warp group
    const int pw = ((N + TPR - 1) / TPR + 1) & ~1;
    const int n0 = min(N, (warp >> 2) * pw), n1 = min(N, n0 + pw);
    const bool live = r < rows;
    double* crow = p.C + (r0 + r) * p.ldc;
    // a chunk of 8 columns inside [n0, n1) is moved as four 16-byte pieces when C's rows allow it
    auto whole = [&](int c0) { return p.vecc && c0 >= n0 && c0 + 8 <= n1; };
    // old C values of a chunk (in place: this row of A, not yet overwritten); issued before the
    // TMEM loads of the chunk before it, so that the global and TMEM latencies overlap
    auto load_c = [&](int c0, double (&cv)[8]) {
      if (p.beta_zero || !live) {
#pragma unroll
        for (int x = 0; x < 8; x++) cv[x] = 0.0;
      } else if (whole(c0)) {
#pragma unroll
        for (int x = 0; x < 8; x += 2) {
          const double2 w = *reinterpret_cast<const double2*>(crow + c0 + x);
          cv[x] = w.x;
          cv[x + 1] = w.y;
        }
      } else {
#pragma unroll
        for (int x = 0; x < 8; x++) {
          const int n = c0 + x;
          cv[x] = (n >= n0 && n < n1) ? crow[n] : 0.0;
        }
      }
    };
    // 128 registers: no room for a second chunk of C, so a chunk's own C loads go out just
    // before its TMEM loads
    constexpr bool AHEAD = false;
    double cold[8], cnext[8];
    if (AHEAD && n0 < n1) load_c(n0 & ~7, cold);
    for (int c0 = (n0 & ~7); c0 < n1; c0 += 8) {
      if (!AHEAD) load_c(c0, cold);
      uint32_t raw[8][8];
#pragma unroll
      for (int L = 0; L < 8; L++) tmem_ld8(tbase + (uint32_t)(L * NM + c0), raw[L]);
      if (AHEAD && c0 + 8 < n1) load_c(c0 + 8, cnext);
      tmem_wait();
      if (live) {
        // all eight columns are formed (columns beyond N hold zero digits and exponent 0) and
        // masked only at the store; beta * C with the dtype test outside the column loop
        const int e = er[r] - 2112 + 32;
        double out[8];
#pragma unroll
        for (int x = 0; x < 8; x++) out[x] = level_value<MP>(raw, x, e + fcol[c0 + x]);
        if (!p.beta_zero) {
          if (!p.cplx) {
#pragma unroll
            for (int x = 0; x < 8; x++) out[x] = fma(p.beta[0], cold[x], out[x]);
          } else {
#pragma unroll
            for (int x = 0; x < 8; x += 2) {  // (re, im) pairs: c0 is a multiple of 8
              const double cr = cold[x], ci = cold[x + 1];
              out[x] = fma(p.beta[0], cr, fma(-p.beta[1], ci, out[x]));
              out[x + 1] = fma(p.beta[0], ci, fma(p.beta[1], cr, out[x + 1]));
            }
          }
        }
        if (whole(c0)) {
#pragma unroll
          for (int x = 0; x < 8; x += 2) *reinterpret_cast<double2*>(crow + c0 + x) = make_double2(out[x], out[x + 1]);
        } else {
#pragma unroll
          for (int x = 0; x < 8; x++) {
            const int n = c0 + x;
            if (n >= n0 && n < n1) crow[n] = out[x];
          }
        }
      }
      if (AHEAD) {
#pragma unroll
        for (int x = 0; x < 8; x++) cold[x] = cnext[x];
      }
    }
  };
  auto wait_mma = [&](int tile_it) -> bool {  // wait until the MMAs of local tile tile_it completed
    const int b = tile_it & 1;
    return mbar_wait_bounded(&bar_mma[b], (uint32_t)((uses[b] - 1) & 1), p.err);
  };

  // A values of the tile being sliced; the next tile's are loaded into the same registers right
  // after slicing (the old values are dead then), so their latency hides behind the epilogue
  double v[PART];
  auto load_tile = [&](int it) {
    const int64_t r1 = (t_begin + it) * ROWS;
    load_row<PART>(p, r1, row, (int)((p.K - r1) < ROWS ? (p.K - r1) : ROWS), m0, v);
  };
  if (nt > 0 && slicer) load_tile(0);
  for (int it = 0; it < nt && !bail; it++) {
    // row exponents: each part of the columns, combined through shared memory
    int* er = erow + ((it & 1) * TPR) * ROWS;
    if (slicer) {
      uint32_t emax = 0;
#pragma unroll
      for (int j = 0; j < PART; j++) emax = max(emax, exp_field(v[j]));
      er[part * ROWS + row] = (int)emax;
    }
    __syncthreads();
    int e_row = er[row];
#pragma unroll
    for (int q2 = 1; q2 < TPS; q2++) e_row = max(e_row, er[q2 * ROWS + row]);
    // the A' buffer is free once the MMAs that read it completed
    if ((p.nabuf == 1 && it > 0) || (p.nabuf == 2 && it > 1)) {
      bool ok = wait_mma(it - p.nabuf);
      if (__syncthreads_or(!ok)) {
        bail = true;
        break;
      }
    }
    unsigned char* A_ = adig + (size_t)(it % p.nabuf) * p.abuf;
#pragma unroll
    for (int o = 0; o < (slicer ? PART / 8 : 0); o++) {
      const int mo = (m0 >> 3) + o;
      if (mo * 8 >= M) {  // zero padding columns: zero digits
#pragma unroll
        for (int pl = 0; pl < DIGITS; pl++)
          *reinterpret_cast<uint4*>(A_ + kmaj(row, (pl * MP + mo * 8) / 8, lbo_a)) = make_uint4(0, 0, 0, 0);
        continue;
      }
      uint32_t dp[4][DIGITS];  // element pairs (0,1), (2,3), (4,5), (6,7) of the octet
#pragma unroll
      for (int q2 = 0; q2 < 4; q2++) {
        uint32_t gha, gla, ghb, glb;
        bool na, nb;
        g_words(v[o * 8 + 2 * q2], (uint32_t)e_row, gha, gla, na);
        g_words(v[o * 8 + 2 * q2 + 1], (uint32_t)e_row, ghb, glb, nb);
        digit_pairs(gha, gla, na, ghb, glb, nb, dp[q2]);
      }
#pragma unroll
      for (int pl = 0; pl < DIGITS; pl++) {
        const int i = 7 - pl;  // 0-based digit index held by plane pl
        *reinterpret_cast<uint4*>(A_ + kmaj(row, (pl * MP + mo * 8) / 8, lbo_a)) =
            make_uint4(dp[0][i], dp[1][i], dp[2][i], dp[3][i]);
      }
    }
    if (tid < ROWS) er[tid] = e_row;  // the epilogue of this tile reads er[r]
    fence_proxy_async_smem();
    // one accumulator: the epilogue of tile it-1 needs no barrier after this tile's slicing (it
    // reads TMEM and C, not A'), so warps go from slicing straight into it; the barrier that
    // ends the epilogue also completes A' for the MMAs
    const bool drain_first = p.ntbuf == 1 && it > 0;
    if (!drain_first) {
      tc_before();
      __syncthreads();
    }
    if (it + 1 < nt && slicer) load_tile(it + 1);  // in flight during the epilogue and the MMAs
    if (drain_first) {  // one accumulator: drain tile it-1 before tile it's MMAs
      if (p.nabuf != 1) {
        bool ok = wait_mma(it - 1);
        if (__syncthreads_or(!ok)) {
          bail = true;
          break;
        }
      }
      tc_after();
      epilogue(it - 1);
      tc_before();
      __syncthreads();
    }
    if (lane == 0 && warp < 4) {  // warp w issues the chains of levels 2 + w and 9 - w (9 K-steps of MP/16)
      tc_after();
      const uint32_t a0 = smem_u32(A_), b0 = smem_u32(bdig);
      const uint32_t dcol = tmem + (uint32_t)((it % p.ntbuf) * 8 * NM);
#pragma unroll
      for (int side = 0; side < 2; side++) {
        const int L = side ? 9 - warp : 2 + warp;
        const int kq = (L - 1) * MP / 16;  // K-steps of 16
        const int ka = (9 - L) * MP / 8;   // first k-octet of A' for this level
        for (int ks = 0; ks < kq; ks++)
          mma_f16(dcol + (uint32_t)((L - 2) * NM), make_desc(a0 + (uint32_t)(ka + 2 * ks) * lbo_a, lbo_a),
                   make_desc(b0 + (uint32_t)(2 * ks) * lbo_b, lbo_b), idesc, ks > 0 ? 1u : 0u);
      }
      mma_commit(&bar_mma[it & 1]);  // one of the four arrivals that complete the tile's phase
    }
    uses[it & 1]++;
    if (p.ntbuf == 2 && it > 0) {  // the previous tile's epilogue overlaps this tile's MMAs
      bool ok = wait_mma(it - 1);
      if (__syncthreads_or(!ok)) {
        bail = true;
        break;
      }
      tc_after();
      epilogue(it - 1);
      tc_before();
      __syncthreads();
    }
  }
  if (!bail && nt > 0) {
    bool ok = wait_mma(nt - 1);
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
  if (Mr > 64 || Nr > 64) {
    // wider products out of place run as passes of real width <= 64: output columns are
    // independent, and the contraction accumulates through beta (the first pass applies beta,
    // later passes add with beta = 1; each pass rounds once more in FP64)
    const int64_t cw = cplx ? 32 : 64, w = cplx ? 2 : 1;
    if (Mr > 128 || Nr > 128 || (const void*)A == (const void*)C) {
      set_error("split precision TSMM: real widths <= 64, or <= 128 out of place");
      return SKINNY_UNSUPPORTED;
    }
    if (autoselect && (K < 8192 || Nr < 8 || Mr < 4 || Mr * Nr < 128)) {
      set_error("split precision TSMM: not selected automatically for this shape");
      return SKINNY_UNSUPPORTED;
    }
    const double one[2] = {1.0, 0.0};
    for (int64_t n0 = 0; n0 < N; n0 += cw)
      for (int64_t m0 = 0; m0 < M; m0 += cw) {
        const skinny_status s = split_tsmm(h, cplx, std::min(cw, M - m0), std::min(cw, N - n0), K, A + w * m0, lda,
                                           alpha, B + w * (n0 * ldb + m0), ldb, m0 == 0 ? beta : (const void*)one,
                                           C + w * n0, ldc, st, false);
        if (s != SKINNY_OK) return s;
      }
    return SKINNY_OK;
  }
  // auto selection (measured on GB300 over every width pair of {1, 2, 4, 8, 16, 32, 64}^2, FP64
  // and complex FP64, ~512 MB of operands), on the real widths (complex doubled): split wins from
  // Mr * Nr >= 128 with Nr >= 8 and a contraction width Mr >= 4 (real 8x16 1.5x, 16x8 1.4x, 4x32
  // 1.2x, 64x8 1.7x, 64x64 9.8x; complex 4x8 1.5x, 32x4 1.65x, 64x64 7.3x); narrower products stay
  // on the CUDA-core kernels (real 8x8 0.83x, 4x16 0.82x, 32x4 0.68x, complex 1x64 0.65x).  The
  // autotuner can override.
  const bool wins = Mr * Nr >= 128 && Nr >= 8 && Mr >= 4;
  if (autoselect && (K < 8192 || !wins)) {
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
  const int MP = Mr <= 16 ? 16 : (Mr <= 32 ? 32 : 64);
  a.NM = Nr <= 16 ? 16 : (Nr <= 32 ? 32 : 64);
  a.cplx = cplx;
  std::memset(a.alpha, 0, sizeof a.alpha);
  std::memset(a.beta, 0, sizeof a.beta);
  std::memcpy(a.alpha, alpha, cplx ? 16 : 8);
  std::memcpy(a.beta, beta, cplx ? 16 : 8);
  a.beta_zero = a.beta[0] == 0.0 && a.beta[1] == 0.0;
  a.inplace = (const void*)A == (const void*)C;
  // in place with M == N: C = A (alpha B + beta I); the epilogue then needs no old C and no FMA
  a.fold = a.inplace && M == N && !a.beta_zero;
  if (a.fold) a.beta_zero = 1;
  a.vec = ((uintptr_t)A % 16 == 0) && (a.lda % 2 == 0);
  a.vecc = ((uintptr_t)C % 16 == 0) && (a.ldc % 2 == 0);
  a.abuf = (uint32_t)(ROWS * 8 * MP * 2);  // 128 rows x 8 planes x MP x fp16
  const int64_t bdig = round_up((int64_t)8 * MP * a.NM * 2, 1024);
  const int64_t avail = h->dev.smem_optin - HDR - bdig;
  a.nabuf = avail >= 2 * (int64_t)a.abuf ? 2 : 1;
  if (avail < (int64_t)a.abuf) {
    set_error("split precision TSMM: tiles do not fit in shared memory");
    return SKINNY_UNSUPPORTED;
  }
  // two CTAs per SM where a CTA fits half the TMEM and half the shared memory (contraction width
  // 16: 128 registers); otherwise one CTA with two accumulator sets where they fit
  const int smem_need = (int)(HDR + bdig + (int64_t)a.nabuf * a.abuf);
  const bool two = MP <= 16 && 8 * a.NM <= 256 && 2 * smem_need <= h->dev.smem_optin;
  a.ntbuf = two ? 256 / (8 * a.NM) : (2 * 8 * a.NM <= 512 ? 2 : 1);
  a.tmem_cols = two ? 256 : (a.ntbuf * 8 * a.NM <= 256 ? 256 : 512);
  a.ntiles = (K + ROWS - 1) / ROWS;
  a.err = h->err;
  const int smem = (int)(HDR + bdig + (int64_t)a.nabuf * a.abuf);
  const int per_sm = two ? 2 : 1;
  int64_t grid = std::min<int64_t>((int64_t)h->dev.sms * per_sm, a.ntiles);
  if (grid < 1) grid = 1;
  cudaError_t e;
  switch (MP) {
    case 16:
      if (two) {
        static SmemAttr attr;
        ensure_smem_attr(split_tsmm_kernel<16, 256>, smem, attr);
        split_tsmm_kernel<16, 256><<<(int)grid, 256, smem, st>>>(a);
      } else {
        static SmemAttr attr;
        ensure_smem_attr(split_tsmm_kernel<16, 512>, smem, attr);
        split_tsmm_kernel<16, 512><<<(int)grid, 512, smem, st>>>(a);
      }
      break;
    case 32: {
      static SmemAttr attr;
      ensure_smem_attr(split_tsmm_kernel<32, 512>, smem, attr);
      split_tsmm_kernel<32, 512><<<(int)grid, 512, smem, st>>>(a);
      break;
    }
    default: {
      static SmemAttr attr;
      ensure_smem_attr(split_tsmm_kernel<64, 512>, smem, attr);
      split_tsmm_kernel<64, 512><<<(int)grid, 512, smem, st>>>(a);
      break;
    }
  }
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("split tsmm launch: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  return SKINNY_OK;
}

}  // namespace skinny
