// split_wide.cu -- FP64 TSMTTSM in split precision for widths 17..128 on tcgen05 tensor cores
// (no counterpart in the reference, whose FP64 TSMTTSM kernels are CUDA-core DFMA loops, e.g.
// tsmttsm/genv5.cuh:28-89; the product and its alpha/beta semantics are those of
// tsmttsm/genv5.cuh:92-98 with the cross-block sum done inside the launch).
//
// From M = N = 32 on, a CUDA-core FP64 TSMTTSM is bound by the FP64 pipe (1.2 TFLOP/s on GB300).
// Here each C block of 64 x 64 is formed from 8-bit digit products on the tensor cores, exactly,
// with every element sliced once.
//
// Scheme:
//   * Per column of A (and of B) a shared exponent E holds for an epoch: an element x is
//     x = sign * F * 2^(E - 1084) with F < 2^62 a fixed-point integer, and F is written as 8
//     balanced base-256 digits d_1..d_8 (d_1 in [-64, 64], the others in [-128, 127]).  The
//     sign is applied to F before splitting, so the digits of a negative x are the digits of -F.
//     When a column meets an element larger than 2^E allows, E is raised (with 4 bits of
//     headroom) and a new epoch starts for the whole CTA.
//   * Digits are exact in FP16.  For a stage of 16 rows the digits are laid out as FP16 planes
//     (K-major, no swizzle): A' holds 12 planes of 64 rows in the order
//     [0, 1, 5 | 0, 2, 6 | 0, 3, 7 | 0, 4, 8] (0 = a zero plane, p = digit p of the 64 columns),
//     so the 128-row window [A_i ; A_{i+4}] is contiguous for i = -3..4; B' holds the planes
//     [0, 1, 2, ..., 8], so the 128-row window [B_j ; B_{j+1}] is contiguous for j = 0..7.
//   * One tcgen05.mma (M = N = 128, K = 16, FP16 x FP16 -> FP32 in TMEM) of window i of A' and
//     window j of B' forms four 64 x 64 quadrants at digit levels (i + j, i + j + 1) in TMEM
//     lanes 0..63 and (i + j + 4, i + j + 5) in lanes 64..127.  Two accumulators
//     collect all 36 digit pairs with level i + j <= 9:
//        key 2:  i = -3..2, j = 2 - i   -> levels 2, 3 (lanes 0-63) and 6, 7 (lanes 64-127)
//        key 4:  i = -3..4, j = 4 - i   -> levels 4, 5 and 8, 9
//     14 MMAs per 16 rows; each pair is counted once.  Levels >= 10 are dropped (weight below
//     2^-56 of the leading level).
//   * A cell of an accumulator sums at most 8 digit products per row (|d d| <= 2^14), so over a
//     period of 128 rows every partial sum is an integer of magnitude < 2^24 and the FP32
//     accumulation is exact.  The two accumulators take 256 TMEM columns; two sets alternate
//     between periods, so the drain of one period runs while the MMAs of the next one proceed.
//   * Drain: TMEM -> int32 -> per C cell one int64 word per lane half (levels 2..5 packed with
//     shifts 24, 16, 8, 0 on lanes 0..63; levels 6..9 on lanes 64..127), summed over the periods
//     of an epoch in registers.  FP64 arithmetic happens only when an epoch ends: the int64 words
//     are converted, scaled by 2^(EA + EB - 2080) (levels 2..5) or 2^(EA + EB - 2112) (6..9) and
//     added to the CTA's FP64 partials.
//   * Warp roles: warps 0-7 slice (one column and 8 rows per thread; 4 rows in Gram mode, where
//     B is A) and drain; warp 8 streams rows of A and B into a ring of FP64 stages with 1-D TMA
//     bulk copies (one per row; 8-byte cp.async where rows are not 16-byte aligned); warp 9
//     issues the MMAs.  Every wait is bounded; a wait that runs
//     out sets the error word and the CTA finishes without waiting further and writes no C.
//   * Blocks of 64 x 64 (M or N > 64) run in the same launch, as do the row chunks of every
//     block; the last CTA of a block (ticket) sums the chunks' partials in chunk order and
//     applies alpha and beta.  Gram (A = B) computes the upper blocks only and mirrors them.
//   * Folded stages (M, N <= 32): a stage holds 32 rows; rows 0..15 fill plane rows 0..31 and
//     rows 16..31 fill plane rows 32..63 (column c of row 16 + r is plane row 32 + c).  The
//     diagonal quadrants of the 64 x 64 accumulators then hold the sums over the two row halves
//     (the off-diagonal quadrants pair different rows and are not read), so a 32-wide product
//     uses every slicer and every MMA column, and the halves are added at the end.
// Inputs must be finite (Inf/NaN have no fixed-point form).
#include <cuda_fp16.h>

#include <atomic>
#include <cstring>

#include "api_internal.h"

namespace skinny {

namespace splitw {

constexpr int ROWS = 16;     // K rows per stage (one MMA K-step)
constexpr int PSTAGES = 8;   // stages per accumulation period (128 rows: exact FP32 sums)
constexpr int DSLOTS = 3;    // digit slots
constexpr int MAXR = 8;      // FP64 stages (at most)
constexpr int HEAD = 4;      // exponent headroom granted when a column's exponent is raised
constexpr int NSL = 256;     // slicer / drain threads (warps 0-7)
constexpr int THREADS = NSL + 64;
constexpr int W = 64;        // block width
constexpr uint32_t LBO_A = 12 * 64 * 16;  // bytes between the two k-octets of A'
constexpr uint32_t LBO_B = 9 * 64 * 16;
constexpr uint32_t SLOT_A = 2 * LBO_A;
constexpr uint32_t SLOT = SLOT_A + 2 * LBO_B;  // 43008
constexpr uint32_t RAW_OP = ROWS * W * 8;      // one operand of an FP64 stage
constexpr int HDR = 4096;
constexpr int MAX_EPOCH_PERIODS = 1 << 14;     // int64 words hold 2^15 periods of < 2^48.1
constexpr int GROUP = 16;                      // chunks per first-level group of the finish (<= 15 groups)

struct Args {
  const void* A;  // FP64, or FP32 (widened exactly when read); the stage ring keeps the type
  const void* B;
  void* C;        // FP64, or FP32 with out_f32
  int64_t K, lda, ldb, ldc;
  int M, N;
  double alpha, beta;
  int beta_zero;
  int nblk, bm, sym;  // 64 x 64 blocks; sym: A == B, upper blocks only
  int bulk;           // rows by bulk copy (16-byte aligned rows of even width)
  int abase16, bbase16;  // A / B start on a 16-byte boundary (dense stages by one bulk copy)
  int rstages;
  uint32_t raw_stage;  // bytes per FP64 stage
  int64_t nstages;     // ceil(K / rows per stage)
  double* partials;    // [nblk][nchunks][2][4096], then [nblk][15][4096] group sums
  unsigned* counter;   // tickets: [nblk][16] (15 groups + the block)
  int* err;
  int out_f32;
};

// A' plane slot of digit plane p (p <= 0: zero planes), for the chain order above
__host__ __device__ constexpr int slot_a(int p) { return 3 * ((p + 3) & 3) + ((p + 3) >> 2); }

__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t lbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;  // k-octet stride
  d |= (uint64_t)(128 >> 4) << 32;              // 8-row-group stride
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
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// bytes a bulk copy will complete on the barrier, without an arrival
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// arrive on the mbarrier once every cp.async of this thread so far has landed
__device__ __forceinline__ void cp_async_arrive(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// named barrier over the 256 slicer threads; returns 1 on every thread if pred holds on any
__device__ __forceinline__ int slicers_any(int pred) {
  int r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.s32 p, %1, 0;\n bar.red.or.pred q, 1, 256, p;\n selp.s32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"(pred)
      : "memory");
  return r;
}
__device__ __forceinline__ void slicers_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

// bounded wait that also gives up as soon as another thread of the CTA has given up; the producer
// and MMA warps sleep between polls so that their polling leaves issue slots to the slicers
__device__ __forceinline__ bool wait_ab(uint64_t* bar, uint32_t parity, volatile int* ab, int* err,
                                        uint32_t sleep_ns = 0) {
  for (uint32_t i = 0; i < (1u << 22); i++) {
    if (mbar_try_wait(bar, parity)) return true;
    if (*ab) return false;
    if (sleep_ns) __nanosleep(sleep_ns);
  }
  *ab = 1;
  if (err) atomicExch(err, SKINNY_DEVERR_TIMEOUT);
  return false;
}

// signed fixed-point value of x relative to exponent field E, offset for balanced base-256 digits
__device__ __forceinline__ uint64_t fixed_g(double x, uint32_t E) {
  const uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  const uint32_t ef = (hi >> 20) & 0x7FF;
  const uint32_t eff = ef ? ef : 1u;
  const uint64_t mant = ((uint64_t)((hi & 0xFFFFFu) | (ef ? 0x100000u : 0u)) << 32) | lo;
  const uint32_t sh = E - eff;  // E >= eff for every nonzero element of the epoch
  uint64_t F = sh < 64 ? ((mant << 9) >> sh) : 0ull;
  if (hi >> 31) F = 0ull - F;
  return F + 0x8080808080808080ull;
}

// FP16 pair (digit of x, digit of y) from the word (byte_x, 0x64, byte_y, 0x64): value 1024 + g
// minus 1152 = g - 128, exact.  t interleaves one 32-bit half of the offset fixed-point values of
// two elements: __byte_perm(x, y, 0x7362) = (x.b2, y.b2, x.b3, y.b3) feeds selectors 0x4342
// (byte 3: the higher digit) and 0x4140 (byte 2); 0x5140 gives bytes 1 and 0 the same way.
__device__ __forceinline__ uint32_t half_pair(uint32_t t, uint32_t sel) {
  uint32_t w = __byte_perm(t, 0x64646464u, sel), d;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(d) : "r"(w), "r"(0x64806480u));
  return d;
}

__device__ __forceinline__ double pow2i(int e) {  // 2^e, clamped to the normal range
  e = e < -1022 ? -1022 : (e > 1023 ? 1023 : e);
  return __hiloint2double((e + 1023) << 20, 0);
}

template <typename TI, bool FOLD>
__global__ void __launch_bounds__(THREADS, 1) split_wide_kernel(const Args p) {
  constexpr uint32_t ES = sizeof(TI);
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* raw_full = reinterpret_cast<uint64_t*>(smem);  // [MAXR]
  uint64_t* raw_empty = raw_full + MAXR;                   // [MAXR]
  uint64_t* dfull = raw_full + 2 * MAXR;                   // [DSLOTS]
  uint64_t* dempty = dfull + 4;                            // [DSLOTS]
  uint64_t* bar_fin = dempty + 4;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 512);
  volatile int* abort_f = reinterpret_cast<volatile int*>(smem + 516);
  volatile int* flags = reinterpret_cast<volatile int*>(smem + 528);  // [DSLOTS]
  int* rec_epoch = reinterpret_cast<int*>(smem + 576);                // [2]
  int* rec = reinterpret_cast<int*>(smem + 1024);                     // [2][128]: EA[64], EB[64]
  int* acc_rec = reinterpret_cast<int*>(smem + 2048);                 // [128]
  unsigned char* dig = smem + HDR;
  unsigned char* raw = dig + DSLOTS * SLOT;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int blk = blockIdx.x % p.nblk, chunk = blockIdx.x / p.nblk, nchunks = gridDim.x / p.nblk;
  int bi, bj;
  if (p.sym) {  // upper triangle, column by column: (0,0), (0,1), (1,1), ...
    int b = blk;
    bj = 0;
    while (b > bj) {
      b -= bj + 1;
      bj++;
    }
    bi = b;
  } else {
    bi = blk % p.bm;
    bj = blk / p.bm;
  }
  const int Mb = min(W, p.M - W * bi), Nb = min(W, p.N - W * bj);
  const TI* Ab = static_cast<const TI*>(p.A) + W * bi;
  const TI* Bb = static_cast<const TI*>(p.sym ? p.A : p.B) + W * bj;
  const int64_t ldb = p.sym ? p.lda : p.ldb;
  const bool gram = p.sym && bi == bj;
  const int64_t s_begin = p.nstages * chunk / nchunks, s_end = p.nstages * (chunk + 1) / nchunks;
  const int nst = (int)(s_end - s_begin);
  const int R = p.rstages;
  // row strides (doubles) of the FP64 stages: dense operands land as one block of rows
  // dense operands (ld == block width, 16-byte aligned start): a stage's rows are one contiguous run
  const bool dense_a = p.abase16 && p.lda == Mb, dense_b = (p.sym ? p.abase16 : p.bbase16) && ldb == Nb;
  // rows per stage; row stride of the stage's rows that are copied one by one (a folded stage
  // holds 32 rows of at most 32 values in the same 16 x 64 space)
  const int SR = FOLD ? 2 * ROWS : ROWS, rw = FOLD ? W / 2 : W;
  const int rsa = dense_a ? Mb : rw, rsb = dense_b ? Nb : rw;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < R; s++) {
      mbar_init(&raw_full[s], p.bulk ? 1 : 32);
      mbar_init(&raw_empty[s], 8);
    }
    for (int s = 0; s < DSLOTS; s++) {
      mbar_init(&dfull[s], 8);
      mbar_init(&dempty[s], 1);
    }
    mbar_init(bar_fin, 1);
    *abort_f = 0;
    fence_mbar_init();
  }
  // zero planes and unused columns stay zero: clear every digit slot once
  for (uint32_t o = tid * 16; o < DSLOTS * SLOT; o += THREADS * 16)
    *reinterpret_cast<uint4*>(dig + o) = make_uint4(0, 0, 0, 0);
  fence_proxy_async_smem();
  tc_before();
  __syncthreads();
  tc_after();
  const uint32_t tmem = *tslot;

  if (warp == 8) {
    // ---- producer: FP64 rows of A and B into the stage ring -------------------------------------
    int issued = 0;
    for (int ls = 0; ls < nst; ls++) {
      const int rs = ls % R, use = ls / R;
      if (use > 0) {
        int ok = 0;
        if (lane == 0) ok = wait_ab(&raw_empty[rs], (uint32_t)((use - 1) & 1), abort_f, p.err, 64);
        if (!__shfl_sync(0xffffffffu, ok, 0)) break;
      }
      const int64_t row0 = (s_begin + ls) * SR;
      const int rows = (int)min((int64_t)SR, p.K - row0);
      TI* dA = reinterpret_cast<TI*>(raw + (size_t)rs * p.raw_stage);
      TI* dB = dA + ROWS * W;
      if (p.bulk) {
        if (lane == 0) mbar_arrive_expect_tx(&raw_full[rs], (uint32_t)(rows * (Mb + (gram ? 0 : Nb)) * ES));
        __syncwarp();
        // dense rows (ld == block width): the stage is one contiguous copy; otherwise one per row
        if (dense_a && lane == 0) bulk_g2s(dA, Ab + row0 * p.lda, (uint32_t)(rows * Mb * ES), &raw_full[rs]);
        if (!gram && dense_b && lane == 1) bulk_g2s(dB, Bb + row0 * ldb, (uint32_t)(rows * Nb * ES), &raw_full[rs]);
        const int na = dense_a ? 0 : rows, nb = (gram || dense_b) ? 0 : rows;
        for (int r = lane; r < na + nb; r += 32) {
          if (r < na)
            bulk_g2s(dA + r * rw, Ab + (row0 + r) * p.lda, (uint32_t)(Mb * ES), &raw_full[rs]);
          else
            bulk_g2s(dB + (r - na) * rw, Bb + (row0 + r - na) * ldb, (uint32_t)(Nb * ES), &raw_full[rs]);
        }
      } else {
        // rows not all 16-byte aligned (odd widths or leading dimensions): a dense operand whose
        // stage starts and ends on 16-byte boundaries (always but for an odd last stage) is one
        // bulk copy, announced on the barrier without an arrival; the rest element by element;
        // one arrival per lane once its element copies have landed
        const bool sa = dense_a && (row0 * Mb * ES) % 16 == 0 && (rows * Mb * ES) % 16 == 0;
        const bool sb = !gram && dense_b && (row0 * Nb * ES) % 16 == 0 && (rows * Nb * ES) % 16 == 0;
        if (lane == 0 && (sa || sb)) {
          mbar_expect_tx(&raw_full[rs], (uint32_t)(((sa ? rows * Mb : 0) + (sb ? rows * Nb : 0)) * ES));
          if (sa) bulk_g2s(dA, Ab + row0 * p.lda, (uint32_t)(rows * Mb * ES), &raw_full[rs]);
          if (sb) bulk_g2s(dB, Bb + row0 * ldb, (uint32_t)(rows * Nb * ES), &raw_full[rs]);
        }
        if (!sa)
          for (int e = lane; e < rows * Mb; e += 32) {
            const int r = e / Mb, c = e - r * Mb;
            if constexpr (ES == 8)
              cp_async8(dA + r * rsa + c, Ab + (row0 + r) * p.lda + c);
            else
              cp_async4(dA + r * rsa + c, Ab + (row0 + r) * p.lda + c);
          }
        if (!gram && !sb)
          for (int e = lane; e < rows * Nb; e += 32) {
            const int r = e / Nb, c = e - r * Nb;
            if constexpr (ES == 8)
              cp_async8(dB + r * rsb + c, Bb + (row0 + r) * ldb + c);
            else
              cp_async4(dB + r * rsb + c, Bb + (row0 + r) * ldb + c);
          }
        cp_async_arrive(&raw_full[rs]);
      }
      issued = ls + 1;
    }
    // copies in flight must land before the CTA ends
    if (!p.bulk) asm volatile("cp.async.wait_all;" ::: "memory");
    if (lane == 0)
      for (int ls = max(0, issued - R); ls < issued; ls++)
        mbar_wait_bounded(&raw_full[ls % R], (uint32_t)((ls / R) & 1), nullptr);
  } else if (warp == 9) {
    // ---- MMA issuer ------------------------------------------------------------------------------
    if (lane == 0) {
      const uint32_t idesc = (1u << 4) | ((128u >> 3) << 17) | ((128u >> 4) << 24);  // F32 <- F16 x F16
      const uint32_t dig0 = smem_u32(dig);
      int issued = 0;
      for (int ls = 0; ls < nst; ls++) {
        const int ds = ls % DSLOTS;
        if (!wait_ab(&dfull[ds], (uint32_t)((ls / DSLOTS) & 1), abort_f, p.err, 32)) break;
        tc_after();
        const int f = flags[ds];
        const uint32_t start = f & 1, buf = (f >> 1) & 1;
        const uint32_t a0 = dig0 + ds * SLOT, b0 = a0 + SLOT_A;
        const uint32_t d0 = tmem + buf * 256;
#pragma unroll
        for (int i = -3; i <= 2; i++)
          mma_f16(d0, desc(a0 + slot_a(i) * 1024, LBO_A), desc(b0 + (2 - i) * 1024, LBO_B), idesc,
                  (start && i == -3) ? 0u : 1u);
#pragma unroll
        for (int i = -3; i <= 4; i++)
          mma_f16(d0 + 128, desc(a0 + slot_a(i) * 1024, LBO_A), desc(b0 + (4 - i) * 1024, LBO_B), idesc,
                  (start && i == -3) ? 0u : 1u);
        mma_commit(&dempty[ds]);
        issued++;
      }
      if (issued) {  // every MMA has finished before the TMEM is released
        mma_commit(bar_fin);
        mbar_wait_bounded(bar_fin, 0, nullptr);
      }
    }
  } else {
    // ---- slicers / drain (warps 0-7) ------------------------------------------------------------
    // slicing unit: column c of A or B and 8 rows (Gram: column c of A and 4 rows).  Lanes are
    // laid out so that a half-warp reads 16 consecutive columns of one row (no bank conflicts)
    // and a quarter-warp stores 128 contiguous bytes of digits.
    const bool isB = !gram && warp >= 4;
    const int c = gram ? 8 * warp + (lane & 7) : 16 * (warp & 3) + (lane & 15);
    const int sub = gram ? (lane >> 3) : (lane >> 4);
    const int nrow = gram ? 4 : 8;
    // folded stages: plane row c holds column c % 32 of the stage's row half c / 32
    const int cact = FOLD ? (c & 31) : c, rbase = FOLD ? ROWS * (c >> 5) : 0;
    const bool cvalid = cact < (isB ? Nb : Mb);
    const int cofs = (c >> 3) * 128 + (c & 7) * 16;  // row c of a digit plane (8-row core groups)
    uint32_t Ecur = 0;
    // drain cells: TMEM lane 32 q + lane (q = warp % 4), C column block [32 nh, 32 nh + 32)
    const int q = warp & 3, nh = warp >> 2;
    const int hm = q >> 1;                  // 0: levels 2..5, 1: levels 6..9
    const int m = (32 * q + lane) & 63;
    // cells this thread keeps: folded stages keep the two diagonal quadrants only
    const bool live = !FOLD || (q & 1) == nh;
    const int mv = FOLD ? (m & 31) : m, nofs = FOLD ? 32 * nh : 0;
    long long acc[32];
#pragma unroll
    for (int x = 0; x < 32; x++) acc[x] = 0;
    int acc_epoch = -1;
    bool flushed = false;
    double* part = p.partials + ((size_t)(blk * nchunks + chunk) * 2 + hm) * 4096;

    auto flush = [&]() {
      const int ea = acc_rec[m];
#pragma unroll
      for (int x = 0; x < 32; x++) {
        const int n = 32 * nh + x;
        if (live && mv < Mb && n - nofs < Nb) {
          double v = 0.0;
          if (acc_epoch >= 0)
            v = (double)acc[x] * pow2i(ea - 1040) * pow2i(acc_rec[64 + n] - 1040 - (hm ? 32 : 0));
          double* d = part + n * 64 + m;
          *d = flushed ? *d + v : v;
        }
        acc[x] = 0;
      }
      flushed = true;
    };
    // drain piece k (cells 8k..8k+7 of this thread) of the TMEM set `buf`; piece 0 first closes
    // the accumulators' epoch when the period belongs to a new one
    auto drain_piece = [&](int buf, int k) {
      if (k == 0) {
        const int ep = rec_epoch[buf];
        if (ep != acc_epoch) {  // uniform: a new epoch begins with this period
          flush();
          slicers_sync();
          if (tid < 128) acc_rec[tid] = rec[buf * 128 + tid];
          slicers_sync();
          acc_epoch = ep;
        }
      }
      tc_after();
      const uint32_t tb = tmem + ((uint32_t)(32 * q) << 16) + buf * 256 + 32 * nh;
#pragma unroll
      for (int hp = 0; hp < 4; hp++) {
        if (hp != k || !live) continue;
        uint32_t s0[8], s1[8], s2[8], s3[8];
        tmem_ld8(tb + hp * 8, s0);          // key 2, columns j   : level 2 / 6
        tmem_ld8(tb + 64 + hp * 8, s1);     // key 2, columns j+1 : level 3 / 7
        tmem_ld8(tb + 128 + hp * 8, s2);    // key 4, columns j   : level 4 / 8
        tmem_ld8(tb + 192 + hp * 8, s3);    // key 4, columns j+1 : level 5 / 9
        tmem_wait_ld();
#pragma unroll
        for (int x = 0; x < 8; x++) {
          const long long l0 = __float2int_rn(__uint_as_float(s0[x]));
          const long long l1 = __float2int_rn(__uint_as_float(s1[x]));
          const long long l2 = __float2int_rn(__uint_as_float(s2[x]));
          const long long l3 = __float2int_rn(__uint_as_float(s3[x]));
          acc[hp * 8 + x] += (l0 << 24) + (l1 << 16) + (l2 << 8) + l3;
        }
      }
      tc_before();
    };

    int cur_buf = 1, pstart = 0, epoch = 0, epoch_periods = 0;
    // the period before the current one is drained in 4 pieces over the stages that follow the
    // completion of its last MMAs, so that the conversions interleave with slicing
    int pend = 0, pend_buf = 0, pend_last = 0, pend_piece = 0;
    for (int ls = 0; ls < nst; ls++) {
      const int rs = ls % R, ds = ls % DSLOTS;
      const int64_t row0 = (s_begin + ls) * SR;
      const int rows = (int)min((int64_t)SR, p.K - row0);
      // lane 0 waits for the FP64 stage (TMA) and for the MMAs that read the digit slot; the
      // warp barrier then orders the other lanes' reads and writes after those waits
      if (lane == 0) {
        wait_ab(&raw_full[rs], (uint32_t)((ls / R) & 1), abort_f, p.err);
        if (ls >= DSLOTS) wait_ab(&dempty[ds], (uint32_t)(((ls / DSLOTS) - 1) & 1), abort_f, p.err);
      }
      __syncwarp();
      // load my unit and its column maximum
      const TI* T = reinterpret_cast<const TI*>(raw + (size_t)rs * p.raw_stage) + (isB ? ROWS * W : 0);
      const int rstr = isB ? rsb : rsa;
      // column maximum of |x| from the high words (the exponent field of the largest high word is
      // the largest exponent field); nonzero low words mark subnormals in an otherwise zero column
      double v[8];
      uint32_t mh = 0, ol = 0;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const int rr = rbase + sub * nrow + k;
        v[k] = (k < nrow && cvalid && rr < rows) ? (double)T[rr * rstr + cact] : 0.0;
        mh = max(mh, (uint32_t)__double2hiint(v[k]) & 0x7FFFFFFFu);
        ol |= (uint32_t)__double2loint(v[k]);
      }
      if (gram) {
        mh = max(mh, __shfl_xor_sync(0xffffffffu, mh, 8));
        ol |= __shfl_xor_sync(0xffffffffu, ol, 8);
      }
      mh = max(mh, __shfl_xor_sync(0xffffffffu, mh, 16));
      ol |= __shfl_xor_sync(0xffffffffu, ol, 16);
      uint32_t e = mh >> 20;
      if (e == 0 && (mh | ol)) e = 1;
      __syncwarp();
      if (lane == 0) mbar_arrive(&raw_empty[rs]);
      const int bump = slicers_any(e > Ecur);
      const bool start = ls == 0 || bump || ls - pstart >= PSTAGES || epoch_periods >= MAX_EPOCH_PERIODS;
      if (start) {
        if (pend) {  // the period before the current one still holds its TMEM set: finish it now
          // its last MMAs: waited on already once its slot was reused (ls >= pend_last + DSLOTS);
          // before that the slot's barrier has not moved past that phase, so the parity wait holds
          if (ls < pend_last + DSLOTS && lane == 0)
            wait_ab(&dempty[pend_last % DSLOTS], (uint32_t)((pend_last / DSLOTS) & 1), abort_f, p.err);
          __syncwarp();
          for (int k = pend_piece; k < 4; k++) drain_piece(pend_buf, k);
          pend = 0;
        }
        if (ls > 0) {
          pend = 1;
          pend_buf = cur_buf;
          pend_last = ls - 1;
          pend_piece = 0;
        }
        cur_buf ^= 1;
        pstart = ls;
        if (bump || ls == 0 || epoch_periods >= MAX_EPOCH_PERIODS) {
          epoch++;
          epoch_periods = 0;
        }
        epoch_periods++;
        if (e > Ecur) Ecur = e + HEAD;
        if (sub == 0) {
          rec[cur_buf * 128 + (isB ? 64 : 0) + c] = (int)Ecur;
          if (gram) rec[cur_buf * 128 + 64 + c] = (int)Ecur;
        }
        if (tid == 0) rec_epoch[cur_buf] = epoch;
      } else if (pend && ls >= pend_last + DSLOTS) {
        // the MMAs of the pending period's last stage are complete (waited on for slot reuse)
        drain_piece(pend_buf, pend_piece);
        if (++pend_piece == 4) pend = 0;
      }
      if (tid == 0) flags[ds] = (start ? 1 : 0) | (cur_buf << 1);
      // slice: digits relative to Ecur into slot ds
      unsigned char* sa = dig + (size_t)ds * SLOT;
      unsigned char* sb = sa + SLOT_A;
      if (cvalid) {
        // digits 2 gi + 1 and 2 gi + 2 of each element pair come from one byte interleave
        if (!gram) {
          uint64_t g[8];
#pragma unroll
          for (int k = 0; k < 8; k++) g[k] = fixed_g(v[k], Ecur);
          unsigned char* dst = (isB ? sb + sub * LBO_B : sa + sub * LBO_A) + cofs;
#pragma unroll
          for (int gi = 0; gi < 4; gi++) {
            uint32_t wa[4], wb[4];
#pragma unroll
            for (int pp = 0; pp < 4; pp++) {
              const uint32_t x = gi < 2 ? (uint32_t)(g[2 * pp] >> 32) : (uint32_t)g[2 * pp];
              const uint32_t y = gi < 2 ? (uint32_t)(g[2 * pp + 1] >> 32) : (uint32_t)g[2 * pp + 1];
              const uint32_t t = __byte_perm(x, y, (gi & 1) ? 0x5140 : 0x7362);
              wa[pp] = half_pair(t, 0x4342);
              wb[pp] = half_pair(t, 0x4140);
            }
            const int d1 = 2 * gi + 1, d2 = 2 * gi + 2;
            *reinterpret_cast<uint4*>(dst + (isB ? d1 : slot_a(d1)) * 1024) = make_uint4(wa[0], wa[1], wa[2], wa[3]);
            *reinterpret_cast<uint4*>(dst + (isB ? d2 : slot_a(d2)) * 1024) = make_uint4(wb[0], wb[1], wb[2], wb[3]);
          }
        } else {
          uint64_t g[4];
#pragma unroll
          for (int k = 0; k < 4; k++) g[k] = fixed_g(v[k], Ecur);
          unsigned char* da = sa + (sub >> 1) * LBO_A + cofs + (sub & 1) * 8;
          unsigned char* db = sb + (sub >> 1) * LBO_B + cofs + (sub & 1) * 8;
#pragma unroll
          for (int gi = 0; gi < 4; gi++) {
            uint32_t wa[2], wb[2];
#pragma unroll
            for (int pp = 0; pp < 2; pp++) {
              const uint32_t x = gi < 2 ? (uint32_t)(g[2 * pp] >> 32) : (uint32_t)g[2 * pp];
              const uint32_t y = gi < 2 ? (uint32_t)(g[2 * pp + 1] >> 32) : (uint32_t)g[2 * pp + 1];
              const uint32_t t = __byte_perm(x, y, (gi & 1) ? 0x5140 : 0x7362);
              wa[pp] = half_pair(t, 0x4342);
              wb[pp] = half_pair(t, 0x4140);
            }
            const int d1 = 2 * gi + 1, d2 = 2 * gi + 2;
            *reinterpret_cast<uint2*>(da + slot_a(d1) * 1024) = make_uint2(wa[0], wa[1]);
            *reinterpret_cast<uint2*>(db + d1 * 1024) = make_uint2(wa[0], wa[1]);
            *reinterpret_cast<uint2*>(da + slot_a(d2) * 1024) = make_uint2(wb[0], wb[1]);
            *reinterpret_cast<uint2*>(db + d2 * 1024) = make_uint2(wb[0], wb[1]);
          }
        }
      }
      fence_proxy_async_smem();
      tc_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&dfull[ds]);
    }
    // last periods
    if (pend) {
      if (nst - 1 < pend_last + DSLOTS && lane == 0)  // no processed stage reused its slot
        wait_ab(&dempty[pend_last % DSLOTS], (uint32_t)((pend_last / DSLOTS) & 1), abort_f, p.err);
      __syncwarp();
      for (int k = pend_piece; k < 4; k++) drain_piece(pend_buf, k);
    }
    if (nst > 0) {
      if (lane == 0)
        wait_ab(&dempty[(nst - 1) % DSLOTS], (uint32_t)(((nst - 1) / DSLOTS) & 1), abort_f, p.err);
      __syncwarp();
      for (int k = 0; k < 4; k++) drain_piece(cur_buf, k);
    }
    flush();
    // the CTA's sum of a cell: levels 2..5 (half 0) plus levels 6..9 (half 1), into half 0; with
    // folded stages the second row half's quadrant is then added to the first's
    slicers_sync();
    if (hm == 0 && live && mv < Mb)
      for (int x = 0; x < 32; x++) {
        const int n = 32 * nh + x;
        if (n - nofs < Nb) part[n * 64 + m] += part[4096 + n * 64 + m];
      }
    if constexpr (FOLD) {
      slicers_sync();
      if (hm == 0 && nh == 0 && q == 0 && m < Mb)
        for (int x = 0; x < Nb; x++) part[x * 64 + m] += part[(x + 32) * 64 + m + 32];
    }
  }

  tc_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
  if (*abort_f) return;

  // ---- cross-CTA finish, two levels: the last CTA of each group of GROUP chunks sums the group's
  // partials in chunk order; the last group to finish sums the group sums in group order and
  // applies alpha and beta (deterministic; the work is spread over the group finishers) -----------
  __threadfence();
  __syncthreads();
  __shared__ int s_last;
  const int ngroups = (nchunks + GROUP - 1) / GROUP, grp = chunk / GROUP;
  const int gsize = min(GROUP, nchunks - grp * GROUP);
  unsigned* gcount = p.counter + blk * 16;  // [grp] per group, [15] for the block
  if (tid == 0) s_last = (atomicAdd(gcount + grp, 1u) == (unsigned)(gsize - 1));
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  const double* P = p.partials + (size_t)blk * nchunks * 8192;           // [chunk][2][4096], half 0 = CTA sum
  double* G = p.partials + (size_t)gridDim.x * 8192 + (size_t)blk * 15 * 4096;  // [group][4096]
  for (int e = tid; e < Mb * Nb; e += THREADS) {
    const int cell = (e / Mb) * 64 + e % Mb;
    double v[GROUP];
#pragma unroll
    for (int i = 0; i < GROUP; i++) v[i] = i < gsize ? __ldcg(P + (size_t)(grp * GROUP + i) * 8192 + cell) : 0.0;
    double sum = 0.0;
#pragma unroll
    for (int i = 0; i < GROUP; i++) sum += v[i];
    G[(size_t)grp * 4096 + cell] = sum;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    gcount[grp] = 0u;
    s_last = (atomicAdd(gcount + 15, 1u) == (unsigned)(ngroups - 1));
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int e = tid; e < Mb * Nb; e += THREADS) {
    const int mm = e % Mb, nn = e / Mb, cell = nn * 64 + mm;
    double v[15];
#pragma unroll
    for (int i = 0; i < 15; i++) v[i] = i < ngroups ? __ldcg(G + (size_t)i * 4096 + cell) : 0.0;
    double sum = 0.0;
#pragma unroll
    for (int i = 0; i < 15; i++) sum += v[i];
    const int64_t ci = (int64_t)(W * bj + nn) * p.ldc + W * bi + mm, cmi = (int64_t)(W * bi + mm) * p.ldc + W * bj + nn;
    const bool mirror = p.sym && bi < bj;  // Gram: the mirrored block holds the same sums
    if (p.out_f32) {  // the one rounding of an FP32 result
      float* C = static_cast<float*>(p.C);
      C[ci] = (float)(p.beta_zero ? p.alpha * sum : (double)C[ci] * p.beta + sum * p.alpha);
      if (mirror) C[cmi] = (float)(p.beta_zero ? p.alpha * sum : (double)C[cmi] * p.beta + sum * p.alpha);
    } else {
      double* C = static_cast<double*>(p.C);
      C[ci] = p.beta_zero ? p.alpha * sum : C[ci] * p.beta + sum * p.alpha;
      if (mirror) C[cmi] = p.beta_zero ? p.alpha * sum : C[cmi] * p.beta + sum * p.alpha;
    }
  }
  if (tid == 0) gcount[15] = 0u;
}

}  // namespace splitw

skinny_status split_wide(skinny_handle h, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                         const void* alpha, const double* B, int64_t ldb, const void* beta, double* C,
                         int64_t ldc, cudaStream_t st) {
  return split_wide_t(h, false, false, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st);
}

skinny_status split_wide_t(skinny_handle h, bool in_f32, bool out_f32, int64_t M, int64_t N, int64_t K,
                           const void* A, int64_t lda, const void* alpha, const void* B, int64_t ldb,
                           const void* beta, void* C, int64_t ldc, cudaStream_t st) {
  using namespace splitw;
  const int64_t es = in_f32 ? 4 : 8;
  if (M > 128 || N > 128) {
    set_error("split precision TSMTTSM: M, N <= 128");
    return SKINNY_UNSUPPORTED;
  }
  Args a;
  a.A = A;
  a.B = B;
  a.C = C;
  a.K = K;
  a.lda = lda;
  a.ldb = ldb;
  a.ldc = ldc;
  a.M = (int)M;
  a.N = (int)N;
  if (out_f32) {  // FP32 scalars widened (exactly)
    float af, bf;
    std::memcpy(&af, alpha, 4);
    std::memcpy(&bf, beta, 4);
    a.alpha = af;
    a.beta = bf;
  } else {
    std::memcpy(&a.alpha, alpha, 8);
    std::memcpy(&a.beta, beta, 8);
  }
  a.out_f32 = out_f32;
  a.beta_zero = a.beta == 0.0;
  a.sym = (A == B) && (lda == ldb) && (M == N);
  a.bm = (int)((M + W - 1) / W);
  const int bn = (int)((N + W - 1) / W);
  a.nblk = a.sym ? a.bm * (a.bm + 1) / 2 : a.bm * bn;
  // bulk copies: 16-byte aligned rows whose block widths are 16-byte multiples
  const int64_t per16 = 16 / es;
  const bool aligned =
      (uintptr_t)A % 16 == 0 && (uintptr_t)B % 16 == 0 && lda % per16 == 0 && ldb % per16 == 0;
  a.bulk = aligned && M % per16 == 0 && N % per16 == 0;
  a.abase16 = (uintptr_t)A % 16 == 0;
  a.bbase16 = (uintptr_t)B % 16 == 0;
  a.raw_stage = (a.sym && a.nblk == 1) ? RAW_OP : 2 * RAW_OP;
  const bool fold = M <= W / 2 && N <= W / 2;  // 32-row stages folded into the 64-row planes
  const int64_t fixed = HDR + (int64_t)DSLOTS * SLOT;
  a.rstages = (int)std::min<int64_t>(MAXR, (h->dev.smem_optin - fixed) / a.raw_stage);
  if (a.rstages < 2) {
    set_error("split precision: stages do not fit in shared memory");
    return SKINNY_UNSUPPORTED;
  }
  const int smem = (int)(fixed + (int64_t)a.rstages * a.raw_stage);
  const int64_t srows = fold ? 2 * ROWS : ROWS;
  a.nstages = (K + srows - 1) / srows;
  const int64_t nchunks = std::max<int64_t>(1, std::min<int64_t>({a.nstages, h->dev.sms / a.nblk,
                                                                   (int64_t)15 * GROUP}));
  const int64_t grid = nchunks * a.nblk;
  Workspace& ws = h->ws[st];
  skinny_status s = workspace_ensure(ws, ((size_t)grid * 2 + (size_t)a.nblk * 15) * 4096 * 8, st);
  if (s != SKINNY_OK) return s;
  a.partials = (double*)ws.partials;
  a.counter = ws.counter;
  a.err = h->err;
  static SmemAttr attr[4];
  auto launch = [&](auto kernel, SmemAttr& at) {
    ensure_smem_attr(kernel, smem, at);
    kernel<<<(int)grid, THREADS, smem, st>>>(a);
  };
  if (!in_f32)
    fold ? launch(split_wide_kernel<double, true>, attr[0]) : launch(split_wide_kernel<double, false>, attr[1]);
  else
    fold ? launch(split_wide_kernel<float, true>, attr[2]) : launch(split_wide_kernel<float, false>, attr[3]);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("split wide tsmttsm launch: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  return SKINNY_OK;
}

}  // namespace skinny
