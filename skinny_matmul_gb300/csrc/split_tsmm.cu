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
//   * Digit-stacked MMAs: for A digit i, one tcgen05.mma (M = 128 rows, K = 16 columns m) against
//     B's digit planes j = 1..9-i stacked along N gives every pair (i, j) with i + j <= 9 at once,
//     written to the accumulator columns of level L = i + j (level L at columns (L-2) NB of a block
//     of NB output columns).  Eight MMAs per 16 columns of the contraction form D_L(r, n) =
//     sum_{i+j=L} sum_m a_i b_j for L = 2..9; levels >= 10 are dropped (weight below 2^-56 of the
//     leading level).  |D_L| <= 2^14 MP (L - 2) (the top digit is at most 64 in magnitude): exact
//     in the FP32 TMEM accumulators.
//   * Epilogue: V = sum_L D_L 2^(8(9-L)) (|V| < 2^74) is formed as a 64-bit integer W = V / 2^12
//     (level_window), rounded to a double (integer instructions, or the FP64 pipe's conversion
//     when there is no beta*C) and scaled by 2^(e_r + f_n - 2100) in the exponent field; beta*C
//     is one FMA.
//   * Warp roles, hand-offs through mbarriers, no CTA-wide barrier while streaming (16 warps):
//       slicers     (8 warps, two threads per row) read the FP64 values of a 128-row tile (the
//                   next tile's are loaded right after a tile is sliced), take the row exponent,
//                   and write the digit planes into an A' stage; warp 0 then issues the tile's
//                   MMAs (one elected lane): per block of NB output columns, 8 MP / 16 MMAs into
//                   one of 2 or 4 TMEM accumulator sets, so that a block's epilogue overlaps the
//                   next blocks' MMAs;
//       epilogue    (8 warps: 2 groups of one warp per TMEM lane quadrant) convert the level
//                   sums; the groups take chunks of 8 output columns in turn; old C values are
//                   prefetched chunk by chunk (cp.async) into a shared-memory ring per group,
//                   several chunks ahead.
//     Every wait is bounded; a wait that runs out sets the error word and every role stops at its
//     next wait (C is then incomplete).
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
constexpr int DIGITS = 8;
constexpr int THREADS = 512;  // 16 warps: four per SM sub-partition, 128 registers
// Warp roles: 8 slicer warps (two threads per row; warp 0 issues the MMAs) and 8 epilogue warps
// (two groups of one warp per TMEM lane quadrant).  Measured and dropped at MP = 16: 4 slicer
// warps (one thread per row) with 12 epilogue warps -- three groups split blocks of 2 or 4 chunks
// unevenly, and the slicers fell behind (real 8 x 32 3.76 -> 4.60 ms, 16 x 16 1.14 -> 1.25 ms).
template <int MP>
__host__ __device__ constexpr int slicer_warps() { return 8; }
template <int MP>
__host__ __device__ constexpr int epi_groups() { return (16 - slicer_warps<MP>()) / 4; }
constexpr int MAXAST = 3;                 // A' stages (at most)
constexpr int CHUNK_BYTES = ROWS * 64;    // one chunk of old C: 8 doubles of each of 128 rows
constexpr uint32_t SLEEP_MMA = 32;        // ns between polls of the MMA thread
// Per contraction width MP: the ring of row-exponent records (tiles), the header (barriers, TMEM
// slot, column exponents, row exponents; a multiple of 1024), and the old-C chunks each epilogue
// warp group keeps in flight.  At MP = 64 B' (64 KB at N = 64) and one A' stage (128 KB) leave
// 35 KB: a 3 KB header and two chunks per group fill the 227 KB exactly.
template <int MP>
__host__ __device__ constexpr int row_ring() { return MP == 64 ? 4 : 8; }
template <int MP>
__host__ __device__ constexpr int hdr_bytes() { return MP == 64 ? 3072 : 5120; }
template <int MP>
__host__ __device__ constexpr int c_depth() { return MP == 64 ? 2 : (MP == 32 ? 3 : 4); }

struct Args {
  const void* A;    // storage type T of the kernel (double or float), as B and C
  const void* B;    // real: B[n*ldb+m]; complex: the complex B (interleaved)
  void* C;
  int64_t K, lda, ldb, ldc;  // in doubles (complex: lda, ldc already doubled; ldb in complex elements)
  int M, N;                  // real widths (complex: 2M, 2N)
  int NM;                    // output width padded: 16, 32 or 64
  int NB, ncb;               // output columns per accumulator block (16 or 32), blocks per tile
  int nsets;                 // TMEM accumulator sets (512 / (8 NB))
  int nast;                  // A' stages
  uint32_t astage;           // bytes of one A' stage (8 planes x 128 rows x MP x FP16)
  uint32_t bbytes;           // bytes reserved for B' (8 planes x NM x MP x FP16, 1024-aligned)
  int cplx;                  // B is complex (alpha, beta complex)
  double alpha[2], beta[2];
  int beta_zero, inplace, vec;  // vec: rows of A may be read as 16-byte pairs
  int fold;                     // beta folded into B's diagonal (in place, M == N); beta_zero then set
  int vecc;                     // rows of C may be read and written as 16-byte pairs
  int64_t ntiles;
  int la;  // MMA issue: 0 by slicer warp 0, else by epilogue warp 8 this many tiles ahead
  int* err;
};

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((128 >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}
// issued by one elected lane of a converged warp, so that the operands stay warp-uniform
__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p, e;\n elect.sync _|e, 0xffffffff;\n setp.ne.b32 p, %4, 0;\n"
      " @e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "{\n .reg .pred e;\n elect.sync _|e, 0xffffffff;\n"
      " @e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n}\n" ::"r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}
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
template <typename T>
__device__ __forceinline__ double alpha_b(const Args& p, int m, int n) {
  if (m >= p.M || n >= p.N) return 0.0;
  const T* B = static_cast<const T*>(p.B);
  if (!p.cplx) {
    const double v = (double)B[(int64_t)n * p.ldb + m] * p.alpha[0];
    return (p.fold && m == n) ? v + p.beta[0] : v;
  }
  const int nc = n >> 1, mc = m >> 1;
  const double br = B[2 * ((int64_t)nc * p.ldb + mc)], bi = B[2 * ((int64_t)nc * p.ldb + mc) + 1];
  double ar = br * p.alpha[0] - bi * p.alpha[1], ai = br * p.alpha[1] + bi * p.alpha[0];
  if (p.fold && mc == nc) {
    ar += p.beta[0];
    ai += p.beta[1];
  }
  return ((n & 1) == 0) ? ((m & 1) == 0 ? ar : -ai) : ((m & 1) == 0 ? ai : ar);
}

// A row values of this thread's part of the columns (HALF values) for tile row r0 + row, widened
// to double (exact for float)
template <int HALF, typename T>
__device__ __forceinline__ void load_row(const Args& p, int64_t r0, int row, int rows, int m0, double (&v)[HALF]) {
  const bool ok = row < rows;
  const T* a = static_cast<const T*>(p.A) + (r0 + row) * p.lda + m0;
  if (ok && p.vec && m0 + HALF <= p.M) {
    if constexpr (sizeof(T) == 8) {
#pragma unroll
      for (int j = 0; j < HALF; j += 2) {
        double2 x = p.inplace ? *reinterpret_cast<const double2*>(a + j) : __ldg(reinterpret_cast<const double2*>(a + j));
        v[j] = x.x;
        v[j + 1] = x.y;
      }
    } else {
#pragma unroll
      for (int j = 0; j < HALF; j += 4) {
        float4 x = p.inplace ? *reinterpret_cast<const float4*>(a + j) : __ldg(reinterpret_cast<const float4*>(a + j));
        v[j] = x.x;
        v[j + 1] = x.y;
        v[j + 2] = x.z;
        v[j + 3] = x.w;
      }
    }
  } else {
#pragma unroll
    for (int j = 0; j < HALF; j++) v[j] = (ok && m0 + j < p.M) ? a[j] : 0.0;
  }
}

// Level sums to integers on the FMA pipe.  An FP32 accumulator holds an exact integer D; for
// |D| <= 2^22, D + 1.5 * 2^23 lies in [2^23, 2^24], where FP32 spacing is 1, so the sum's bit
// pattern is 0x4B400000 + D.  For |D| < 2^24 the same with 1.5 * 2^25 (spacing 4) gives D's
// multiple of 4, h, and D - h (|D - h| <= 2) follows exactly; with 1.5 * 2^24 (spacing 2) the
// pattern 0x4BC00000 + D / 2 gives D to within 1.  (A float-to-int conversion instruction runs on
// GB300's narrow FP64 pipe, and integer bit manipulation on the ALU pipe, which the rest of the
// epilogue keeps busy.)
__device__ __forceinline__ int f32_int22(float f) { return __float_as_int(f + 12582912.0f) - 0x4B400000; }
__device__ __forceinline__ int f32_int24(float f) {
  const float t = f + 50331648.0f;  // 1.5 * 2^25
  const float h = t - 50331648.0f;  // exact: D's nearest multiple of 4
  return 4 * (__float_as_int(t) - 0x4C400000) + f32_int22(f - h);
}
__device__ __forceinline__ int f32_int23_near(float f) { return 2 * (__float_as_int(f + 25165824.0f) - 0x4BC00000); }

// The product of a row and a column from the eight FP32 level sums in raw[L][x] (exact integers
// D_2..D_9 of V = sum_L D_L 2^(8(9-L))) is V * 2^(er + fc - 2112) for row and column exponent
// fields er and fc.  level_window forms W = V / 2^12 as a 64-bit integer:
//   * Sizes: the top digit is at most 64 in magnitude, the others 128, so |D_2| <= 2^12 MP and
//     |D_L| <= 2^14 MP (L - 2) for L >= 3.  At MP <= 32 every level is within 2^22; at MP = 64
//     levels 2..6 are, level 7 (< 2^23) is converted exactly in two steps, and levels 8 and 9
//     (weights 2^8 and 1 in V) to within 1, which the 2^12 that W drops below covers.
//   * Pairs P = D_L * 256 + D_{L+1} fit 32 bits (|P| < 2^31 for every pair), and |V| < 2^74 (V is
//     the exact sum of MP products of 62-bit fixed-point values, shifted down by 2^56), so
//     W = P1 2^36 + P2 2^20 + P3 2^4 + floor(P4 / 2^12) is a 64-bit integer (|W| < 2^62) within
//     one unit of V / 2^12.  Dropping those 12 bits keeps W relative to the largest possible V at
//     2^-62, below the fixed-point truncation of the inputs themselves.
// The double W * 2^(er + fc - 2100) then comes from one of two finishers (same accuracy): the
// integer one runs on the ALU pipe, the conversion one on the FP64 pipe, which is free for it
// when the epilogue has no beta FMA.  W == 0 and results below the normal range give 0.
// A pair of levels within 2^22 takes one multiply-add on the magic-number bit patterns: with
// b = 0x4B400000 + D, b0 * 256 + b1 = D0 * 256 + D1 + 0x8B400000 modulo 2^32 (0x4B400000 * 256 is
// 0x40000000 modulo 2^32), and |D0 * 256 + D1| < 2^31 makes the signed difference exact.
__device__ __forceinline__ int pair22(float f0, float f1) {
  const uint32_t b0 = __float_as_uint(f0 + 12582912.0f), b1 = __float_as_uint(f1 + 12582912.0f);
  return (int)(b0 * 256u + b1 - 0x8B400000u);
}
template <int MP, int W>
__device__ __forceinline__ long long level_window(const uint32_t (&raw)[8][W], int x) {
  float f[8];
#pragma unroll
  for (int L = 0; L < 8; L++) f[L] = __uint_as_float(raw[L][x]);
  const int P1 = pair22(f[0], f[1]), P2 = pair22(f[2], f[3]);
  int P3, P4;
  if constexpr (MP <= 32) {
    P3 = pair22(f[4], f[5]);
    P4 = pair22(f[6], f[7]);
  } else {
    P3 = f32_int22(f[4]) * 256 + f32_int24(f[5]);
    P4 = f32_int23_near(f[6]) * 256 + f32_int23_near(f[7]);
  }
  return ((long long)P1 << 36) + (long long)P2 * (1 << 20) + (long long)P3 * 16 + (long long)(P4 >> 12);
}
// Integer finisher, ex = er + fc - 1014 (the biased exponent field of the result when W has its
// leading one at bit 63): normalise |W| so that its leading one is bit 63, round on bit 10 (ties
// away from zero), and add the exponent field below the leading one, so that a mantissa carry
// raises the exponent.
__device__ __forceinline__ double window_int(long long W, int ex) {
  const uint32_t sgn = (uint32_t)((unsigned long long)W >> 32) & 0x80000000u;
  const unsigned long long m = (unsigned long long)(W < 0 ? -W : W);
  const int z = __clzll((long long)m);                       // 64 for W == 0
  const unsigned long long n = m << (z & 63);                 // leading one at bit 63 (0 for W == 0)
  const unsigned long long r = (n >> 11) + ((n >> 10) & 1);  // 53 bits, or 2^53 after a carry
  const int ef = ex - z;                                      // biased exponent field of the result
  const uint32_t hi = ((uint32_t)(ef - 1) << 20) + (uint32_t)(r >> 32);
  const bool ok = n != 0 && ef > 0;
  return __hiloint2double(ok ? (int)(hi | sgn) : 0, ok ? (int)(uint32_t)r : 0);
}
// Conversion finisher, es = er + fc - 2100: the FP64 pipe's int64 -> double conversion (rounded
// to nearest; exact scaling follows), then es added to the exponent field.
__device__ __forceinline__ double window_cvt(long long W, int es) {
  const double d = __ll2double_rn(W);
  const int hi = __double2hiint(d), lo = __double2loint(d);
  const int e0 = (hi >> 20) & 0x7FF;  // 0 only for W == 0
  const bool ok = e0 != 0 && e0 + es > 0;
  return __hiloint2double(ok ? (int)((uint32_t)hi + ((uint32_t)es << 20)) : 0, ok ? lo : 0);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// bounded wait that also gives up as soon as another thread of the CTA has given up; sleep_ns
// between polls for the MMA thread, which waits most of the time
__device__ __forceinline__ bool wait_ab(uint64_t* bar, uint32_t parity, volatile int* ab, int* err,
                                        uint32_t sleep_ns = 0) {
  for (uint32_t i = 0; i < kWaitPolls; i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*ab) return false;
    if (sleep_ns) __nanosleep(sleep_ns);
  }
  *ab = 1;
  if (err) atomicExch(err, SKINNY_DEVERR_TIMEOUT);
  return false;
}
// asynchronous global -> shared copies of old C (src_bytes < size zero-fills the rest; 0 reads nothing)
__device__ __forceinline__ void cp_async16(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, uint32_t src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <int MP, typename T>
__global__ void __launch_bounds__(THREADS, 1) split_tsmm_kernel(const Args p) {
  constexpr int NSL = slicer_warps<MP>(), NEP = 16 - NSL, EG = epi_groups<MP>();
  constexpr int TPS = NSL * 32 / ROWS;  // slicer threads per row (1 or 2)
  constexpr int PART = MP / TPS;        // A values per slicer thread
  constexpr int CD = c_depth<MP>();    // old-C chunks in flight per epilogue thread
  constexpr int RE = row_ring<MP>(), HDR = hdr_bytes<MP>();
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* afull = reinterpret_cast<uint64_t*>(smem);          // [MAXAST] A' stage written
  uint64_t* aempty = reinterpret_cast<uint64_t*>(smem + 32);    // [MAXAST] its MMAs completed
  uint64_t* tfull = reinterpret_cast<uint64_t*>(smem + 64);     // [4] accumulator set complete
  uint64_t* tempty = reinterpret_cast<uint64_t*>(smem + 96);    // [4] accumulator set read
  uint64_t* efull = reinterpret_cast<uint64_t*>(smem + 128);    // [RE] row exponents written
  uint64_t* eempty = reinterpret_cast<uint64_t*>(smem + 192);   // [RE] row exponents read
  uint64_t* mfin = reinterpret_cast<uint64_t*>(smem + 256);     // every MMA of the CTA completed
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 264);
  volatile int* abort_f = reinterpret_cast<volatile int*>(smem + 268);
  int* fcol = reinterpret_cast<int*>(smem + 512);               // [64] column exponents
  int* erow = reinterpret_cast<int*>(smem + 1024);              // [RE][ROWS] row exponents
  unsigned char* bdig = smem + HDR;                             // B' (1024-aligned)
  unsigned char* adig = bdig + p.bbytes;                        // A' stages
  unsigned char* cbuf = adig + (size_t)p.nast * p.astage;       // [EG groups][CD][ROWS][8 doubles] old C
  const int M = p.M, N = p.N, NB = p.NB;
  // B' per block of NB output columns: rows j * NB + n (digit j + 1 of column n), K-major over
  // m in octets of 8 rows x 16 bytes (no swizzle); bytes between k-octets and between blocks:
  const uint32_t bko = 128u * (uint32_t)NB, bcb = (uint32_t)(MP / 8) * bko;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t t_begin = p.ntiles * blockIdx.x / gridDim.x;
  const int64_t t_end = p.ntiles * (blockIdx.x + 1) / gridDim.x;
  const int nt = (int)(t_end - t_begin);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < MAXAST; s++) {
      mbar_init(&afull[s], NSL);
      mbar_init(&aempty[s], 1);
    }
    for (int k = 0; k < 4; k++) {
      mbar_init(&tfull[k], 1);
      mbar_init(&tempty[k], NEP);
    }
    for (int e = 0; e < RE; e++) {
      mbar_init(&efull[e], NSL);
      mbar_init(&eempty[e], NEP);
    }
    mbar_init(mfin, 1);
    *abort_f = 0;
    fence_mbar_init();
  }
  // ---- B' = digits of alpha * B: column exponents, then (n, m-octet) units -------------------
  if (tid < p.NM) {
    uint32_t f = 0;
    for (int m = 0; m < M; m++) f = max(f, exp_field(alpha_b<T>(p, m, tid)));
    fcol[tid] = (int)f;
  }
  __syncthreads();
  for (int u = tid; u < p.NM * (MP / 8); u += THREADS) {
    const int n = u % p.NM, mo = u / p.NM;
    float d[8][DIGITS];
    bool ng[8];
#pragma unroll
    for (int q2 = 0; q2 < 8; q2++) digits_of(alpha_b<T>(p, mo * 8 + q2, n), (uint32_t)fcol[n], d[q2], ng[q2]);
    unsigned char* bcol = bdig + (uint32_t)(n / NB) * bcb;
#pragma unroll
    for (int j = 0; j < DIGITS; j++) {
      uint4 w = make_uint4(pack2(d[0][j], d[1][j], ng[0], ng[1]), pack2(d[2][j], d[3][j], ng[2], ng[3]),
                           pack2(d[4][j], d[5][j], ng[4], ng[5]), pack2(d[6][j], d[7][j], ng[6], ng[7]));
      *reinterpret_cast<uint4*>(bcol + kmaj(j * NB + n % NB, mo, bko)) = w;
    }
  }
  fence_proxy_async_smem();
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *tslot;

  // MMA issue by one warp, converged, one elected lane: per block of NB output columns, digit
  // i + 1 of A against B planes 0 .. 7 - i (kind::f16, FP16 A and B, FP32 accumulators,
  // M = 128, N = (8 - i) NB) into the next accumulator set.  The issuing warp is slicer warp 0
  // (after it has sliced its rows of the tile) or, where the epilogue has slack (no beta FMA, no
  // old C, few MMAs per tile) and the accumulator sets allow p.la >= 1 tiles of lookahead,
  // epilogue warp 8 (tile t + la before it drains tile t).
  int mjob = 0;
  auto issue_tile = [&](int it) -> bool {
    const int s = it % p.nast;
    if (!wait_ab(&afull[s], (uint32_t)((it / p.nast) & 1), abort_f, p.err, SLEEP_MMA)) return false;
    tc_after();
    const uint32_t as = smem_u32(adig) + (uint32_t)s * p.astage;
    for (int cb = 0; cb < p.ncb; cb++, mjob++) {
      const int k = mjob % p.nsets;
      if (mjob >= p.nsets) {
        if (!wait_ab(&tempty[k], (uint32_t)((mjob / p.nsets - 1) & 1), abort_f, p.err, SLEEP_MMA)) return false;
        tc_after();
      }
      const uint32_t dcol = tmem + (uint32_t)(k * 8 * NB);
      const uint32_t bb = smem_u32(bdig) + (uint32_t)cb * bcb;
#pragma unroll
      for (int ks = 0; ks < MP / 16; ks++)
#pragma unroll
        for (int i = 0; i < DIGITS; i++)
          mma_f16(dcol + (uint32_t)(i * NB), make_desc(as + (uint32_t)(i * MP * 256 + ks * 4096), 2048u),
                  make_desc(bb + (uint32_t)(2 * ks) * bko, bko),
                  (1u << 4) | ((uint32_t)(((DIGITS - i) * NB) >> 3) << 17) | ((128u >> 4) << 24),
                  (ks | i) ? 1u : 0u);
      mma_commit(&tfull[k]);
    }
    mma_commit(&aempty[s]);
    return true;
  };
  if (warp < NSL) {
    // ---- slicers: row = tid / 2, columns [m0, m0 + PART) ------------------------------------
    const int row = tid / TPS, part = tid % TPS, m0 = part * PART;
    double v[PART];
    auto load_tile = [&](int it) {
      const int64_t r1 = (t_begin + it) * ROWS;
      load_row<PART, T>(p, r1, row, (int)((p.K - r1) < ROWS ? (p.K - r1) : ROWS), m0, v);
    };
    if (nt > 0) load_tile(0);
    for (int it = 0; it < nt; it++) {
      const int s = it % p.nast, es = it % RE;
      uint32_t emax = 0;
#pragma unroll
      for (int j = 0; j < PART; j++) emax = max(emax, exp_field(v[j]));
      if (TPS == 2) emax = max(emax, (uint32_t)__shfl_xor_sync(0xffffffffu, emax, 1));
      bool ok = *abort_f == 0;
      if (ok && it >= RE) ok = wait_ab(&eempty[es], (uint32_t)((it / RE - 1) & 1), abort_f, p.err);
      if (ok && it >= p.nast) ok = wait_ab(&aempty[s], (uint32_t)((it / p.nast - 1) & 1), abort_f, p.err);
      if (!__all_sync(0xffffffffu, ok)) break;  // the whole warp leaves together
      if (part == 0) erow[es * ROWS + row] = (int)emax;
      unsigned char* A_ = adig + (size_t)s * p.astage;
#pragma unroll
      for (int o = 0; o < PART / 8; o++) {
        const int mo = (m0 >> 3) + o;
        if (mo * 8 >= M) {  // zero padding columns: zero digits
#pragma unroll
          for (int pl = 0; pl < DIGITS; pl++)
            *reinterpret_cast<uint4*>(A_ + (uint32_t)(pl * MP * 256) + kmaj(row, mo, 2048u)) = make_uint4(0, 0, 0, 0);
          continue;
        }
        uint32_t dp[4][DIGITS];  // element pairs (0,1), (2,3), (4,5), (6,7) of the octet
#pragma unroll
        for (int q2 = 0; q2 < 4; q2++) {
          uint32_t gha, gla, ghb, glb;
          bool na, nb;
          g_words(v[o * 8 + 2 * q2], emax, gha, gla, na);
          g_words(v[o * 8 + 2 * q2 + 1], emax, ghb, glb, nb);
          digit_pairs(gha, gla, na, ghb, glb, nb, dp[q2]);
        }
        // plane pl holds digit pl + 1: 128 rows x MP columns, k-octets 2048 bytes apart
#pragma unroll
        for (int pl = 0; pl < DIGITS; pl++)
          *reinterpret_cast<uint4*>(A_ + (uint32_t)(pl * MP * 256) + kmaj(row, mo, 2048u)) =
              make_uint4(dp[0][pl], dp[1][pl], dp[2][pl], dp[3][pl]);
      }
      fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(&efull[es]);
        mbar_arrive(&afull[s]);
      }
      if (it + 1 < nt) load_tile(it + 1);  // in flight while this tile's MMAs run
      // a wait that runs out sets the abort flag, which the slicers see at the next tile
      if (warp == 0 && p.la == 0) issue_tile(it);
    }
    if (warp == 0 && p.la == 0) {
      mma_commit(mfin);  // completes once every MMA issued by the elected lanes has
      mbar_wait_bounded(mfin, 0, nullptr);
    }
    __syncwarp();
  } else {
    // ---- epilogue: warp NSL + 4 g + q of group g reads TMEM lanes 32q..32q+31 (rows of the tile)
    const int q = warp & 3, r = 32 * q + lane, eg = (warp - NSL) >> 2;
    const int CH = (N + 7) >> 3;        // chunks of 8 output columns per row
    const int CHg = (CH - eg + EG - 1) / EG;  // chunks c = eg, eg + EG, .. of this warp per tile
    const int cpb = NB >> 3;            // chunks per block (even)
    const bool need_c = !p.beta_zero;
    // the FP64-pipe finisher where the epilogue runs no beta FMA on that pipe (measured: with the
    // FMA, the conversion makes the FP64 pipe the bottleneck even on one warp group)
    const bool cvt = !need_c;
    // old C prefetch cursor: this warp's next chunk (tile pf_it, chunk pf_c) goes to ring slot
    // pf_g % CD; one commit group per chunk (empty past the last chunk)
    int pf_it = 0, pf_c = eg, pf_g = 0;
    auto issue = [&]() {
      if (pf_it < nt && CHg > 0) {
        const int c = pf_c;
        const int64_t rr = (t_begin + pf_it) * ROWS + r;
        const bool live = rr < p.K;
        const T* src = static_cast<const T*>(p.C) + rr * p.ldc + 8 * c;
        unsigned char* dst = cbuf + (size_t)(eg * CD + pf_g % CD) * CHUNK_BYTES + r * 64;
        constexpr int PER16 = 16 / (int)sizeof(T);  // elements per 16-byte piece
        if (p.vecc) {
#pragma unroll
          for (int x = 0; x < 8 / PER16; x++) {
            const int left = N - (8 * c + PER16 * x);
            const uint32_t bytes = live && left > 0 ? (uint32_t)(min(left, PER16) * (int)sizeof(T)) : 0u;
            cp_async16(dst + 16 * x, bytes ? (const void*)(src + PER16 * x) : p.C, bytes);
          }
        } else {
#pragma unroll
          for (int x = 0; x < 8; x++) {
            const uint32_t bytes = (live && 8 * c + x < N) ? (uint32_t)sizeof(T) : 0u;
            if constexpr (sizeof(T) == 8)
              cp_async8(dst + 8 * x, bytes ? (const void*)(src + x) : p.C, bytes);
            else
              cp_async4(dst + 4 * x, bytes ? (const void*)(src + x) : p.C, bytes);
          }
        }
        pf_c += EG;
        if (pf_c >= CH) {
          pf_c = eg;
          pf_it++;
        }
      }
      cp_async_commit();
      pf_g++;
    };
    if (need_c)
      for (int i = 0; i < CD - 1; i++) issue();
    const bool issuer = p.la > 0 && warp == NSL;
    if (issuer)
      for (int j = 0; j < p.la && j < nt; j++) issue_tile(j);
    int g = 0;  // this warp's chunks consumed so far
    int job = 0;
    bool ok = true;
    for (int it = 0; it < nt && ok; it++) {
      const int es = it % RE;
      if (issuer && it + p.la < nt) issue_tile(it + p.la);  // a timeout sets the abort flag
      const int64_t rr = (t_begin + it) * ROWS + r;
      const bool live = rr < p.K;
      ok = wait_ab(&efull[es], (uint32_t)((it / RE) & 1), abort_f, p.err);
      if (!__all_sync(0xffffffffu, ok)) {
        ok = false;
        break;
      }
      const int e = erow[es * ROWS + r] - 1014;
      __syncwarp();
      if (lane == 0) mbar_arrive(&eempty[es]);
      T* crow = static_cast<T*>(p.C) + rr * p.ldc;
      for (int cb = 0; cb < p.ncb; cb++, job++) {
        const int k = job % p.nsets;
        ok = wait_ab(&tfull[k], (uint32_t)((job / p.nsets) & 1), abort_f, p.err);
        if (!__all_sync(0xffffffffu, ok)) {
          ok = false;
          break;
        }
        tc_after();
        const uint32_t tb = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(k * 8 * NB);
        const int c_hi = min(CH, (cb + 1) * cpb);
        // this warp's chunks of the block: c = eg (mod EG)
        for (int c = cb * cpb + ((eg - cb * cpb) % EG + EG) % EG; c < c_hi; c += EG, g++) {
          if (need_c) issue();  // chunk g + CD - 1, into the slot of chunk g - 1, read in full already
          // the chunk in two halves of 4 columns: half the TMEM values live at a time, so that the
          // conversion chains of a half fit the registers side by side
          const unsigned char* cs = cbuf + (size_t)(eg * CD + g % CD) * CHUNK_BYTES + r * 64;
          if (need_c) cp_async_wait<CD - 1>();  // this thread's copies of chunk g have landed
#pragma unroll
          for (int hh = 0; hh < 2; hh++) {
            uint32_t raw[8][4];
#pragma unroll
            for (int L = 0; L < 8; L++) tmem_ld4(tb + (uint32_t)(L * NB + 8 * (c - cb * cpb) + 4 * hh), raw[L]);
            double cold[4];
            if (need_c) {
              if constexpr (sizeof(T) == 8) {
                const double2 w0 = reinterpret_cast<const double2*>(cs)[2 * hh];
                const double2 w1 = reinterpret_cast<const double2*>(cs)[2 * hh + 1];
                cold[0] = w0.x;
                cold[1] = w0.y;
                cold[2] = w1.x;
                cold[3] = w1.y;
              } else {
                const float4 w = reinterpret_cast<const float4*>(cs)[hh];
                cold[0] = w.x;
                cold[1] = w.y;
                cold[2] = w.z;
                cold[3] = w.w;
              }
            }
            tmem_wait();
            if (live) {
              // all four columns are formed (columns beyond N hold zero digits and exponent 0)
              // and masked only at the store
              const int c0 = 8 * c + 4 * hh;
              const int4 f = *reinterpret_cast<const int4*>(fcol + c0);
              const int fc[4] = {f.x, f.y, f.z, f.w};
              double out[4];
              if (cvt) {
#pragma unroll
                for (int x = 0; x < 4; x++) out[x] = window_cvt(level_window<MP>(raw, x), e + fc[x] - 1086);
              } else {
#pragma unroll
                for (int x = 0; x < 4; x++) out[x] = window_int(level_window<MP>(raw, x), e + fc[x]);
              }
              if (need_c) {
                if (!p.cplx || p.beta[1] == 0.0) {  // a real beta scales both parts of a complex C alike
#pragma unroll
                  for (int x = 0; x < 4; x++) out[x] = fma(p.beta[0], cold[x], out[x]);
                } else {
#pragma unroll
                  for (int x = 0; x < 4; x += 2) {  // (re, im) pairs: c0 is a multiple of 4
                    const double cr = cold[x], ci = cold[x + 1];
                    out[x] = fma(p.beta[0], cr, fma(-p.beta[1], ci, out[x]));
                    out[x + 1] = fma(p.beta[0], ci, fma(p.beta[1], cr, out[x + 1]));
                  }
                }
              }
              if (p.vecc && c0 + 4 <= N) {
                if constexpr (sizeof(T) == 8) {
                  *reinterpret_cast<double2*>(crow + c0) = make_double2(out[0], out[1]);
                  *reinterpret_cast<double2*>(crow + c0 + 2) = make_double2(out[2], out[3]);
                } else {  // the one rounding of an FP32 result
                  *reinterpret_cast<float4*>(crow + c0) = make_float4((float)out[0], (float)out[1], (float)out[2], (float)out[3]);
                }
              } else {
#pragma unroll
                for (int x = 0; x < 4; x++)
                  if (c0 + x < N) crow[c0 + x] = (T)out[x];
              }
            }
          }
        }
        tc_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&tempty[k]);
      }
    }
    if (need_c) cp_async_wait<0>();
    if (issuer) {
      mma_commit(mfin);
      mbar_wait_bounded(mfin, 0, nullptr);
    }
  }
  tc_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

}  // namespace stsmm

skinny_status split_tsmm_t(skinny_handle h, bool cplx, bool f32, int64_t M, int64_t N, int64_t K, const void* A,
                           int64_t lda, const void* alpha, const void* B, int64_t ldb, const void* beta, void* C,
                           int64_t ldc, cudaStream_t st, bool autoselect) {
  using namespace stsmm;
  const int64_t Mr = cplx ? 2 * M : M, Nr = cplx ? 2 * N : N;
  const int64_t es = f32 ? 4 : 8;  // bytes of a real storage element
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
    const float onef[2] = {1.0f, 0.0f};
    const char *a8 = static_cast<const char*>(A), *b8 = static_cast<const char*>(B);
    char* c8 = static_cast<char*>(C);
    for (int64_t n0 = 0; n0 < N; n0 += cw)
      for (int64_t m0 = 0; m0 < M; m0 += cw) {
        const skinny_status s = split_tsmm_t(
            h, cplx, f32, std::min(cw, M - m0), std::min(cw, N - n0), K, a8 + w * m0 * es, lda, alpha,
            b8 + w * (n0 * ldb + m0) * es, ldb, m0 == 0 ? beta : (f32 ? (const void*)onef : (const void*)one),
            c8 + w * n0 * es, ldc, st, false);
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
  // complex 4 x 4 (real 8 x 8) joined after the warp-role rebuild: 2.0 vs 2.5 ms at 1 GiB of A
  const bool wins = (Mr * Nr >= 128 || (cplx && Mr * Nr >= 64)) && Nr >= 8 && Mr >= 4;
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
  if (f32) {  // FP32 scalars widened (exactly)
    float af[2] = {0.0f, 0.0f}, bf[2] = {0.0f, 0.0f};
    std::memcpy(af, alpha, cplx ? 8 : 4);
    std::memcpy(bf, beta, cplx ? 8 : 4);
    a.alpha[0] = af[0], a.alpha[1] = af[1], a.beta[0] = bf[0], a.beta[1] = bf[1];
  } else {
    std::memcpy(a.alpha, alpha, cplx ? 16 : 8);
    std::memcpy(a.beta, beta, cplx ? 16 : 8);
  }
  a.beta_zero = a.beta[0] == 0.0 && a.beta[1] == 0.0;
  a.inplace = (const void*)A == (const void*)C;
  // in place with M == N: C = A (alpha B + beta I); the epilogue then needs no old C and no FMA
  a.fold = a.inplace && M == N && !a.beta_zero;
  if (a.fold) a.beta_zero = 1;
  a.vec = ((uintptr_t)A % 16 == 0) && ((a.lda * es) % 16 == 0);
  a.vecc = ((uintptr_t)C % 16 == 0) && ((a.ldc * es) % 16 == 0);
  a.NB = a.NM == 16 ? 16 : 32;
  a.ncb = a.NM / a.NB;
  a.nsets = 512 / (8 * a.NB);
  a.astage = (uint32_t)(ROWS * DIGITS * MP * 2);
  a.bbytes = (uint32_t)round_up((int64_t)2 * DIGITS * MP * a.NM, 1024);
  const int HDR = MP == 64 ? hdr_bytes<64>() : (MP == 32 ? hdr_bytes<32>() : hdr_bytes<16>());
  const int64_t cbytes =
      (int64_t)(MP == 64 ? epi_groups<64>() * c_depth<64>()
                         : (MP == 32 ? epi_groups<32>() * c_depth<32>() : epi_groups<16>() * c_depth<16>())) *
      CHUNK_BYTES;
  // the deepest A' ring that fits beside B' and the old-C rings (one stage at MP = 64)
  a.nast = 0;
  for (int ns = MAXAST; ns >= 1 && a.nast == 0; ns--)
    if (HDR + (int64_t)a.bbytes + (int64_t)ns * a.astage + cbytes <= h->dev.smem_optin) a.nast = ns;
  if (a.nast == 0) {
    set_error("split precision TSMM: tiles do not fit in shared memory");
    return SKINNY_UNSUPPORTED;
  }
  a.ntiles = (K + ROWS - 1) / ROWS;
  // without old C the epilogue has slack: it issues the MMAs, la tiles ahead, where the sets allow
  // and a tile takes few MMAs (contraction width 16: 8; measured slower at 32, whose 16 MMAs per
  // tile hold the issuing epilogue warp too long)
  a.la = (a.beta_zero && MP == 16 && a.nsets >= 2 * a.ncb) ? a.nsets / a.ncb - 1 : 0;
  a.err = h->err;
  const int smem = (int)(HDR + (int64_t)a.bbytes + (int64_t)a.nast * a.astage + cbytes);
  int64_t grid = std::min<int64_t>((int64_t)h->dev.sms, a.ntiles);
  if (grid < 1) grid = 1;
  static SmemAttr attr[6];
  auto launch = [&](auto kern, SmemAttr& at) {
    const bool ok = ensure_smem_attr(kern, smem, at);
    if (ok) kern<<<(int)grid, THREADS, smem, st>>>(a);
    return ok;
  };
  bool attr_ok;
  if (!f32) {
    attr_ok = MP == 16 ? launch(split_tsmm_kernel<16, double>, attr[0])
              : MP == 32 ? launch(split_tsmm_kernel<32, double>, attr[1])
                         : launch(split_tsmm_kernel<64, double>, attr[2]);
  } else {
    attr_ok = MP == 16 ? launch(split_tsmm_kernel<16, float>, attr[3])
              : MP == 32 ? launch(split_tsmm_kernel<32, float>, attr[4])
                         : launch(split_tsmm_kernel<64, float>, attr[5]);
  }
  if (!attr_ok) return SKINNY_DEVICE_ERROR;  // the error text is set
  count_launch();
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("split tsmm launch: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  return SKINNY_OK;
}

skinny_status split_tsmm(skinny_handle h, bool cplx, int64_t M, int64_t N, int64_t K, const double* A,
                         int64_t lda, const void* alpha, const double* B, int64_t ldb, const void* beta, double* C,
                         int64_t ldc, cudaStream_t st, bool autoselect) {
  return split_tsmm_t(h, cplx, false, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, autoselect);
}

}  // namespace skinny
