// split.cu -- FP64 TSMTTSM in split precision on tcgen05 tensor cores for M, N <= 16 (no
// counterpart in the reference, whose FP64 kernels are CUDA-core DFMA loops, e.g.
// tsmttsm/genv5.cuh:28-89).  Wider products go to split_wide.cu.
//
// Why: GB300 executes 595 G FP64 FMA/s but 2.25 P FP16 / BF16 tensor flop/s.  A CUDA-core FP64
// TSMTTSM is FP64-bound for every M = N >= 2.  Here each FP64 product is computed exactly from
// 8-bit pieces on the tensor cores, and FP64 arithmetic is used only a few times per 1024 rows.
//
// Scheme (Ozaki-style error-free splitting, written for this kernel):
//   * Per column m of A (and n of B) a shared exponent E holds for an epoch: each element x is a
//     62-bit fixed-point integer F = |x| * 2^(1084 - E) written as 8 balanced base-256 digits
//     d_1..d_8 (d_1 most significant): x = sign * sum_i d_i 2^(8(8-i)) 2^(E-1084).  Digits are
//     exact in FP16 (byte permutes, digits.cuh).  When a round of rows holds an element above
//     2^E's range, that column's E is raised with HEAD bits of headroom and a new period starts.
//   * Digit planes are stacked along the MMA dimensions: A rows (i-1)*MP + m, B rows
//     (j-1)*NP + n, so one tcgen05.mma (M = 128, N = 8*NP, K = 16, FP16 x FP16 -> FP32 in TMEM)
//     forms every digit-pair product d_i(a) d_j(b) for 16 rows of K.
//   * |d_i d_j| <= 2^14, so over a period of <= 1024 rows every partial sum is an integer of
//     magnitude <= 2^24: the FP32 accumulation in TMEM is exact.  Two accumulator sets alternate
//     between periods, so the drain of one period runs while the MMAs of the next proceed.
//   * Drain: TMEM -> int32; level sums S_L = sum_{i+j=L} D_ij (L = 2..9) are formed with a
//     per-lane rotation and warp shuffles (all eight levels per shuffle stage), then in shared
//     memory with integer atomics;
//     V = sum_L S_L 2^(8(16-L)) is assembled from two int64 words and added to an FP64
//     accumulator per C entry with weight 2^(EA+EB-2168).  Levels L >= 10 are dropped: their
//     weight is below 2^-56 of the leading level (2^-52 with the headroom).
//   * Warp roles, hand-offs through mbarriers (no CTA-wide barrier while streaming):
//       warps 0-7  slicers: per round of rr rows (rr * (M + N) / 8 units of one column and 8 rows,
//                  at most two per thread) read the FP64 values from the stage ring (or from
//                  global memory where rows are not 16-byte aligned), check them against the
//                  column exponents (one named barrier per round; two more only when a period
//                  starts), slice them into a digit stage;
//       warps 8-11 drain: one TMEM lane quadrant each;
//       warp 12    producer: whole rounds of rows by 1-D TMA bulk copies into the FP64 ring;
//       warp 13    MMA issuer: rr/16 MMAs per round into the period's accumulator set.
//     The roles that wait most of the time (drain, producer, MMA) sleep between polls, so that
//     their polling leaves issue slots to the slicers.  Every wait is bounded; a wait that runs
//     out sets the error word, every role stops at its next wait, and the CTA writes no C.
//   * Cross-CTA finish in two levels: CTA partials in FP64; the last CTA of each group of 16
//     (ticket) sums its group in CTA order, the last group sums the group sums in group order
//     and applies alpha/beta (deterministic).
// Inputs must be finite (Inf/NaN have no fixed-point form).

#include <cstring>

#include "api_internal.h"
#include "digits.cuh"

namespace skinny {

namespace split {

constexpr int PERIOD = 1024;   // rows accumulated exactly in TMEM (|sum| <= 1024 * 2^14)
constexpr int DIGITS = 8;
constexpr int NSLICE = 8;      // slicer warps 0-7
constexpr int NDRAIN = 4;      // drain warps 8-11 (one TMEM lane quadrant each)
constexpr int WPROD = NSLICE + NDRAIN, WMMA = WPROD + 1;
constexpr int THREADS = (WMMA + 1) * 32;  // 448
constexpr int SLICERS = NSLICE * 32;
constexpr int HEAD = 2;        // exponent headroom granted when a column's exponent is raised
constexpr int MAXST = 4;       // FP64 stages (at most)
constexpr int MAXDST = 3;      // digit stages (at most)
constexpr int DPAD = 128 * 16; // slack after an A digit buffer: the MMA reads 128 rows per k-octet
constexpr int HDR = 2048;      // barriers, TMEM slot, round and period records, exponents
constexpr int SBYTES = 8 * 16 * 16 * 4;  // level sums S[8][16][16]
constexpr int CBYTES = 256 * 8;          // FP64 accumulators of the C entries
constexpr int STATIC_RESERVE = 1024;     // the kernel's static shared memory
constexpr uint32_t SLEEP_DRAIN = 256;    // ns between polls of the drain warps (a period is ~8 rounds)
constexpr uint32_t SLEEP_PRODUCER = 64;  // ns between polls of the producer warp
constexpr uint32_t SLEEP_MMA = 32;       // ns between polls of the MMA thread
constexpr int GROUP = 16;                // CTAs per first-level group of the cross-CTA finish
constexpr int MAXGROUPS = 16;            // groups at most (grid <= 256); counter[MAXGROUPS] is the last level's

struct Args {
  const void* A;  // FP64, or FP32 with in_f32 (widened exactly when read)
  const void* B;
  void* C;        // FP64, or FP32 with out_f32
  int64_t K, lda, ldb, ldc;
  int M, N, MP, NP;  // padded widths (powers of two); NP = MP in Gram mode
  double alpha, beta;
  int beta_zero, gram, bulk;
  int stages, dstages;   // FP64 stages, digit stages
  int rr;                // rows per round (a multiple of 128, <= PERIOD)
  int64_t nrounds;
  uint32_t stage_bytes;  // FP64 stage: rr rows of A (tile_a bytes), then rr rows of B
  uint32_t tile_a;
  int nmma;              // MMA N (multiple of 16, >= 16)
  int tmem_cols;         // two accumulator sets of nmma columns
  uint32_t lbo_a, lbo_b; // bytes between k-octets of the A / B digit buffers
  uint32_t dig_a, dig_b; // bytes of one A / B digit buffer (A includes DPAD)
  double* partials;
  unsigned* counter;
  int* err;
  int out_f32;
};

__device__ __forceinline__ uint64_t make_desc(uint32_t saddr, uint32_t lbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;  // K-direction core-matrix stride
  d |= (uint64_t)((128 >> 4) & 0x3FFF) << 32;  // 8-row-group stride
  d |= (uint64_t)1 << 46;                      // descriptor version
  return d;                                    // no swizzle
}

__device__ __forceinline__ void mma_f16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

template <int X>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, uint32_t (&r)[X]);
template <>
__device__ __forceinline__ void tmem_ld<1>(uint32_t taddr, uint32_t (&r)[1]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r[0]) : "r"(taddr));
}
template <>
__device__ __forceinline__ void tmem_ld<2>(uint32_t taddr, uint32_t (&r)[2]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(taddr));
}
template <>
__device__ __forceinline__ void tmem_ld<4>(uint32_t taddr, uint32_t (&r)[4]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(taddr));
}
template <>
__device__ __forceinline__ void tmem_ld<8>(uint32_t taddr, uint32_t (&r)[8]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// exponent field used for the shared exponent: 0 for zero, 1 for subnormals
__device__ __forceinline__ uint32_t exp_field(double x) {
  uint32_t hi = (uint32_t)__double2hiint(x), lo = (uint32_t)__double2loint(x);
  uint32_t ef = (hi >> 20) & 0x7FF;
  bool nz = ((hi & 0x7FFFFFFFu) | lo) != 0;
  return nz ? (ef ? ef : 1u) : 0u;
}

__device__ __forceinline__ double pow2i(int e) {  // 2^e for e in [-1022, 1023], clamped outside
  e = e < -1022 ? -1022 : (e > 1023 ? 1023 : e);
  return __hiloint2double((e + 1023) << 20, 0);
}

// Slice one unit: 8 consecutive rows (octet o) of column c into the digit buffer `buf`
// (rows (i-1)*CP + c), relative to exponent E.  FP16 digits formed from the bytes of G with byte
// permutes and one HFMA2 per digit pair (digits.cuh).
__device__ __forceinline__ void slice_unit(const double (&v)[8], uint32_t E, int c, int CP, int o,
                                           uint32_t lbo, unsigned char* buf) {
  uint32_t dp[4][NDIGITS];  // row pairs (0,1), (2,3), (4,5), (6,7) of the octet
#pragma unroll
  for (int q = 0; q < 4; q++) {
    uint32_t gha, gla, ghb, glb;
    bool na, nb;
    g_words(v[2 * q], E, gha, gla, na);
    g_words(v[2 * q + 1], E, ghb, glb, nb);
    digit_pairs(gha, gla, na, ghb, glb, nb, dp[q]);
  }
#pragma unroll
  for (int i = 0; i < DIGITS; i++) {
    const int r = i * CP + c;
    *reinterpret_cast<uint4*>(buf + o * lbo + (r >> 3) * 128 + (r & 7) * 16) =
        make_uint4(dp[0][i], dp[1][i], dp[2][i], dp[3][i]);
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// named barriers over one role's threads; return 1 on every thread if pred holds on any
__device__ __forceinline__ int slicers_any(int pred) {
  int r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.s32 p, %1, 0;\n bar.red.or.pred q, 1, 256, p;\n selp.s32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"(pred)
      : "memory");
  return r;
}
__device__ __forceinline__ int drainers_any(int pred) {
  int r;
  asm volatile(
      "{\n .reg .pred p, q;\n setp.ne.s32 p, %1, 0;\n bar.red.or.pred q, 2, 128, p;\n selp.s32 %0, 1, 0, q;\n}\n"
      : "=r"(r)
      : "r"(pred)
      : "memory");
  return r;
}
__device__ __forceinline__ void drainers_sync() { asm volatile("bar.sync 2, 128;" ::: "memory"); }

// Sum of c[t] over the lanes that hold the same column m of A (lane = (i0, m), MP lanes per
// digit): xor-shuffles at distances MP..16, the eight levels' shuffles of a stage issued together
// so that their latencies overlap.
__device__ __forceinline__ void level_reduce(int (&c)[DIGITS], int MP) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    if (o >= MP) {  // warp-uniform
#pragma unroll
      for (int t = 0; t < DIGITS; t++) c[t] += __shfl_xor_sync(0xffffffffu, c[t], o);
    }
  }
}

// bounded wait that also gives up as soon as another thread of the CTA has given up; sleep_ns
// between polls for the roles that wait most of the time
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

template <int NP, typename TI>
__global__ void __launch_bounds__(THREADS, 1) split_tsmttsm_kernel(const Args p) {
  constexpr int BN = NP < 8 ? NP : 8;  // B columns per drain block
  constexpr int NB = NP / BN;          // drain blocks
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);           // [MAXST] FP64 stage landed
  uint64_t* empty = full + MAXST;                                // [MAXST] FP64 stage consumed
  uint64_t* dfull = reinterpret_cast<uint64_t*>(smem + 64);      // [MAXDST] digit stage written
  uint64_t* dempty = reinterpret_cast<uint64_t*>(smem + 96);     // [MAXDST] its MMAs completed
  uint64_t* pdone = reinterpret_cast<uint64_t*>(smem + 128);     // [2] a period's MMAs completed
  uint64_t* pfin = reinterpret_cast<uint64_t*>(smem + 144);      // [2] a period's record published
  uint64_t* drained = reinterpret_cast<uint64_t*>(smem + 160);   // [2] a set's drain finished
  uint64_t* bar_fin = reinterpret_cast<uint64_t*>(smem + 176);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 192);
  volatile int* abort_f = reinterpret_cast<volatile int*>(smem + 196);
  volatile int* rinfo = reinterpret_cast<volatile int*>(smem + 208);  // [MAXDST] period | first << 30
  volatile int* plast = reinterpret_cast<volatile int*>(smem + 224);  // [2] the period is the last
  int* Ecur = reinterpret_cast<int*>(smem + 256);                      // [32] A columns, then B
  int* pe = reinterpret_cast<int*>(smem + 384);                        // [2][32] a period's exponents
  int* S = reinterpret_cast<int*>(smem + HDR);
  double* cacc = reinterpret_cast<double*>(smem + HDR + SBYTES);
  unsigned char* ring = smem + HDR + SBYTES + CBYTES;
  unsigned char* dig = ring + (size_t)p.stages * p.stage_bytes;  // 1024-aligned by the host
  auto digA = [&](int d) { return dig + (size_t)d * (p.dig_a + p.dig_b); };
  auto digB = [&](int d) { return p.gram ? digA(d) : digA(d) + p.dig_a; };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int M = p.M, N = p.N, MP = p.MP;
  const int chunk = blockIdx.x, nchunks = gridDim.x;
  const int64_t t_begin = p.nrounds * chunk / nchunks;
  const int64_t t_end = p.nrounds * (chunk + 1) / nchunks;
  const int nt = (int)(t_end - t_begin);
  const int DST = p.dstages;
  // a round is bulk-copied when its rows end before the last row of the operand starts
  auto is_bulk = [&](int64_t t) { return p.bulk && (t + 1) * (int64_t)p.rr < p.K; };

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tslot)),
                 "r"(p.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int s = 0; s < p.stages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], NSLICE);
    }
    for (int d = 0; d < DST; d++) {
      mbar_init(&dfull[d], NSLICE);
      mbar_init(&dempty[d], 1);
    }
    for (int i = 0; i < 2; i++) {
      mbar_init(&pdone[i], 1);
      mbar_init(&pfin[i], 1);
      mbar_init(&drained[i], 1);
    }
    mbar_init(bar_fin, 1);
    *abort_f = 0;
    fence_mbar_init();
  }
  if (tid < 32) Ecur[tid] = 0;
  for (int e = tid; e < SBYTES / 4; e += THREADS) S[e] = 0;
  for (int e = tid; e < CBYTES / 8; e += THREADS) cacc[e] = 0.0;
  // padding rows of the digit stages stay zero: clear every stage once
  for (uint32_t o = tid * 16; o < (uint32_t)DST * (p.dig_a + p.dig_b); o += THREADS * 16)
    *reinterpret_cast<uint4*>(dig + o) = make_uint4(0, 0, 0, 0);
  fence_proxy_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == WPROD) {
    // ---- producer: whole rounds of rows of A and B into the FP64 stage ring ----------------------
    int issued = 0;
    for (int t = 0; t < nt; t++) {
      const int s = t % p.stages, use = t / p.stages;
      if (use > 0) {
        int ok = 0;
        if (lane == 0) ok = wait_ab(&empty[s], (uint32_t)((use - 1) & 1), abort_f, p.err, SLEEP_PRODUCER);
        if (!__shfl_sync(0xffffffffu, ok, 0)) break;
      }
      if (lane == 0) {
        const int64_t tt = t_begin + t;
        if (is_bulk(tt)) {
          const int64_t r0 = tt * p.rr;
          constexpr uint32_t ES = sizeof(TI);
          const uint32_t ba = (uint32_t)(p.rr * p.lda * ES), bb = p.gram ? 0u : (uint32_t)(p.rr * p.ldb * ES);
          unsigned char* st = ring + (size_t)s * p.stage_bytes;
          mbar_arrive_expect_tx(&full[s], ba + bb);
          bulk_g2s(st, static_cast<const TI*>(p.A) + r0 * p.lda, ba, &full[s]);
          if (!p.gram) bulk_g2s(st + p.tile_a, static_cast<const TI*>(p.B) + r0 * p.ldb, bb, &full[s]);
        } else {
          mbar_arrive(&full[s]);  // no copy: the slicers read this round from global memory
        }
      }
      issued = t + 1;
    }
    // copies in flight land before the CTA ends
    if (lane == 0)
      for (int t = max(0, issued - p.stages); t < issued; t++)
        mbar_wait_bounded(&full[t % p.stages], (uint32_t)((t / p.stages) & 1), nullptr);
  } else if (warp == WMMA) {
    // ---- MMA issuer -------------------------------------------------------------------------------
    if (lane == 0) {
      // idesc: D f32, A/B f16, K-major both, N = nmma, M = 128
      const uint32_t idesc = (1u << 4) | ((uint32_t)(p.nmma >> 3) << 17) | ((128u >> 4) << 24);
      const uint32_t lbb = p.gram ? p.lbo_a : p.lbo_b;
      int pcur = -1, issued = 0;
      bool ok = true;
      for (int t = 0; t < nt; t++) {
        const int d = t % DST;
        if (!wait_ab(&dfull[d], (uint32_t)((t / DST) & 1), abort_f, p.err, SLEEP_MMA)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const int info = rinfo[d];
        const int pp = info & 0x3FFFFFFF;
        const bool first = (info >> 30) & 1;
        if (first) {
          if (pp >= 1) {  // the previous period is complete once its MMAs finish
            mma_commit(&pdone[(pp - 1) & 1]);
            plast[(pp - 1) & 1] = 0;
            mbar_arrive(&pfin[(pp - 1) & 1]);
          }
          if (pp >= 2) {  // this period's accumulator set was drained (period pp - 2)
            if (!wait_ab(&drained[pp & 1], (uint32_t)(((pp - 2) >> 1) & 1), abort_f, p.err, SLEEP_MMA)) {
              ok = false;
              break;
            }
            tc_fence_after();
          }
        }
        const uint32_t a0 = smem_u32(digA(d)), b0 = smem_u32(digB(d));
        const uint32_t dcol = tmem + (uint32_t)((pp & 1) * p.nmma);
        const int ksteps = p.rr / 16;
        for (int ks = 0; ks < ksteps; ks++)
          mma_f16(dcol, make_desc(a0 + 2 * ks * p.lbo_a, p.lbo_a), make_desc(b0 + 2 * ks * lbb, lbb), idesc,
                   (first && ks == 0) ? 0u : 1u);
        mma_commit(&dempty[d]);
        pcur = pp;
        issued++;
      }
      if (ok && pcur >= 0) {
        mma_commit(&pdone[pcur & 1]);
        plast[pcur & 1] = 1;
        mbar_arrive(&pfin[pcur & 1]);
      }
      if (issued) {  // every MMA has finished before the TMEM is released
        mma_commit(bar_fin);
        mbar_wait_bounded(bar_fin, 0, nullptr);
      }
    }
  } else if (warp >= NSLICE) {
    // ---- drain: a period's TMEM set -> level sums -> FP64 accumulators ---------------------------
    const int q = warp - NSLICE;        // TMEM lane quadrant
    const int dtid = tid - SLICERS;     // 0..127
    const int r = 32 * q + lane;        // TMEM lane = A digit row
    const int i0 = r / MP, m = r - i0 * MP;  // digit index (0-based) and column of A
    const bool rvalid = (i0 < DIGITS) && (m < M);
    for (int pp = 0; nt > 0; pp++) {  // K = 0: no rounds, no periods
      const int set = pp & 1;
      const uint32_t par = (uint32_t)((pp >> 1) & 1);
      // one lane per warp polls (sleeping in between); the warp follows
      int ok = 1;
      if (lane == 0) {
        ok = wait_ab(&pfin[set], par, abort_f, p.err, SLEEP_DRAIN);
        if (ok) ok = wait_ab(&pdone[set], par, abort_f, p.err, SLEEP_DRAIN);
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (drainers_any(!ok)) break;
      tc_fence_after();
      const bool last = plast[set] != 0;
      // quadrants holding no digit row (8 * MP <= 32 q) have nothing to drain
      for (int nb = 0; nb < (32 * q < DIGITS * MP ? NB : 0); nb++) {
        uint32_t raw[DIGITS][BN];
#pragma unroll
        for (int j = 0; j < DIGITS; j++) {
          uint32_t tmp[BN];
          tmem_ld<BN>(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(set * p.nmma + j * NP + nb * BN), tmp);
#pragma unroll
          for (int x = 0; x < BN; x++) raw[j][x] = tmp[x];
        }
        tmem_wait_ld();
#pragma unroll
        for (int x = 0; x < BN; x++) {
          const int n = nb * BN + x;
          int R[DIGITS];
#pragma unroll
          // exact (|sum| <= 2^24); the conversion pipe is otherwise idle, the ALU pipe is the slicers'
          for (int j = 0; j < DIGITS; j++) R[j] = rvalid ? __float2int_rn(__uint_as_float(raw[j][x])) : 0;
          // rotate so that R[t] holds the pair (i0+1, j) of level t+2, i.e. j-1 = t - i0
#pragma unroll
          for (int b = 1; b < DIGITS; b <<= 1) {
            if (i0 & b) {
              int T[DIGITS];
#pragma unroll
              for (int t = 0; t < DIGITS; t++) T[t] = R[(t - b + DIGITS) % DIGITS];
#pragma unroll
              for (int t = 0; t < DIGITS; t++) R[t] = T[t];
            }
          }
          int c[DIGITS];
#pragma unroll
          for (int t = 0; t < DIGITS; t++) c[t] = (i0 <= t) ? R[t] : 0;
          level_reduce(c, MP);
          if (lane < MP && rvalid && n < N) {
#pragma unroll
            for (int t = 0; t < DIGITS; t++) atomicAdd(&S[(t * 16 + m) * 16 + n], c[t]);
          }
        }
      }
      tc_fence_before();
      drainers_sync();
      for (int e = dtid; e < M * N; e += NDRAIN * 32) {
        const int mm = e % M, nn = e / M;
        long long sv[8];
#pragma unroll
        for (int t = 0; t < 8; t++) sv[t] = S[(t * 16 + mm) * 16 + nn];
        const long long vhi = (sv[0] << 24) + (sv[1] << 16) + (sv[2] << 8) + sv[3];
        const long long vlo = (sv[4] << 24) + (sv[5] << 16) + (sv[6] << 8) + sv[7];
        const int ea = pe[set * 32 + mm], eb = pe[set * 32 + (p.gram ? nn : 16 + nn)];
        const double v = fma((double)vlo, 0x1p-32, (double)vhi);  // in units of 2^(EA+EB-2080)
        cacc[e] = fma(v * pow2i(ea - 1040), pow2i(eb - 1040), cacc[e]);
      }
      drainers_sync();
      for (int e = dtid; e < SBYTES / 4; e += NDRAIN * 32) S[e] = 0;  // before the next period's atomics
      if (dtid == 0) mbar_arrive(&drained[set]);
      if (last) break;
    }
  } else {
    // ---- slicers: one unit = one column and 8 rows; A units first, then B units ------------------
    const int NUA = (p.rr / 8) * MP;
    const int NUB = p.gram ? 0 : (p.rr / 8) * NP;
    const int NU = NUA + NUB;  // <= 2 * SLICERS (host guarantees)
    int ucol[2], uoct[2], uop[2];
    bool uval[2];
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int u = tid + k * SLICERS;
      if (u < NUA) {
        uop[k] = 0;
        ucol[k] = u % MP;
        uoct[k] = u / MP;
        uval[k] = ucol[k] < M;
      } else {
        const int v = u - NUA;
        uop[k] = 1;
        ucol[k] = v % NP;
        uoct[k] = v / NP;
        uval[k] = u < NU && ucol[k] < N;
      }
    }
    int Ereg[2] = {0, 0};
    int pp = -1, period_rows = 0;
    for (int t = 0; t < nt; t++) {
      const int s = t % p.stages, d = t % DST;
      const int64_t tt = t_begin + t;
      const int64_t r0 = tt * p.rr;
      const int rows = (int)((p.K - r0) < p.rr ? (p.K - r0) : p.rr);
      const bool ok = wait_ab(&full[s], (uint32_t)((t / p.stages) & 1), abort_f, p.err);
      const bool blk = is_bulk(tt);
      const TI* stA = reinterpret_cast<const TI*>(ring + (size_t)s * p.stage_bytes);
      const TI* stB = p.gram ? stA : reinterpret_cast<const TI*>(ring + (size_t)s * p.stage_bytes + p.tile_a);
      double v[2][8];
      uint32_t eu[2] = {0u, 0u};
      bool exceed = false;
      // The 8 rows of an octet o are visited in the order q ^ (o & 7), the same for A and B (a
      // permutation of k inside a k-octet leaves the MMA's sum unchanged): lanes of a half-warp
      // holding different octets then read different banks of the FP64 stage.
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const bool isB = uop[k] != 0;
        const int64_t ld = isB ? p.ldb : p.lda;
        const int g = uoct[k] & 7;
        if (blk) {  // shared-memory stage
          const TI* src = isB ? stB : stA;
#pragma unroll
          for (int q2 = 0; q2 < 8; q2++) {
            const int rr = uoct[k] * 8 + (q2 ^ g);
            v[k][q2] = (ok && uval[k]) ? (double)src[rr * ld + ucol[k]] : 0.0;
          }
        } else {  // global memory (rows not 16-byte aligned, or the last round)
          const TI* src = static_cast<const TI*>(isB ? p.B : p.A) + r0 * ld;
#pragma unroll
          for (int q2 = 0; q2 < 8; q2++) {
            const int rr = uoct[k] * 8 + (q2 ^ g);
            v[k][q2] = (ok && uval[k] && rr < rows) ? (double)src[rr * ld + ucol[k]] : 0.0;
          }
        }
        // largest exponent field of the unit (1 if only subnormals, 0 if all zero): the largest
        // high word without its sign bit gives the field; an OR of the magnitudes tells zero
        uint32_t hmax = 0u, nz = 0u;
#pragma unroll
        for (int q2 = 0; q2 < 8; q2++) {
          const uint32_t h = (uint32_t)__double2hiint(v[k][q2]) & 0x7FFFFFFFu;
          hmax = max(hmax, h);
          nz |= h | (uint32_t)__double2loint(v[k][q2]);
        }
        eu[k] = hmax >> 20;
        if (eu[k] == 0u && nz != 0u) eu[k] = 1u;
        if (uval[k] && (int)eu[k] > Ereg[k]) exceed = true;
      }
      const bool newp = pp < 0 || period_rows + p.rr > PERIOD || exceed;
      bool first = false;
      if (slicers_any(!ok || newp)) {
        if (slicers_any(!ok)) break;
        // a new period: raise the exponents of the columns that met larger elements
#pragma unroll
        for (int k = 0; k < 2; k++)
          if (uval[k] && (int)eu[k] > Ereg[k]) atomicMax(&Ecur[uop[k] * 16 + ucol[k]], (int)eu[k] + HEAD);
        pp++;
        bool ok2 = true;  // the period's exponent slot and accumulator set held period pp - 2
        if (pp >= 2) ok2 = wait_ab(&drained[pp & 1], (uint32_t)(((pp - 2) >> 1) & 1), abort_f, p.err);
        if (slicers_any(!ok2)) break;  // also orders the atomics before the reads below
        if (tid < 32) pe[(pp & 1) * 32 + tid] = Ecur[tid];
#pragma unroll
        for (int k = 0; k < 2; k++) Ereg[k] = uval[k] ? Ecur[uop[k] * 16 + ucol[k]] : 0;
        period_rows = 0;
        first = true;
      }
      // the FP64 stage is consumed: the values are in registers
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      int okd = 1;  // the digit stage is free once the MMAs of round t - DST completed
      if (t >= DST) {
        if (lane == 0) okd = wait_ab(&dempty[d], (uint32_t)(((t / DST) - 1) & 1), abort_f, p.err);
        okd = __shfl_sync(0xffffffffu, okd, 0);
      }
      if (okd) {
#pragma unroll
        for (int k = 0; k < 2; k++)
          if (uval[k]) {
            if (uop[k])
              slice_unit(v[k], (uint32_t)Ereg[k], ucol[k], NP, uoct[k], p.lbo_b, digB(d));
            else
              slice_unit(v[k], (uint32_t)Ereg[k], ucol[k], MP, uoct[k], p.lbo_a, digA(d));
          }
        if (tid == 0) rinfo[d] = pp | (first ? (1 << 30) : 0);
        fence_proxy_async_smem();
        __syncwarp();
        if (lane == 0) mbar_arrive(&dfull[d]);
      }
      period_rows += p.rr;
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.tmem_cols));
  if (*abort_f) return;  // timeout recorded in the error word; no partial, no ticket

  // ---- cross-CTA finish, two levels: the last CTA of each group of GROUP CTAs sums the group's
  // partials in CTA order, the last group to finish sums the group sums in group order and applies
  // alpha and beta (deterministic; each level is one round of independent loads) -----------------
  const int MN = M * N;
  if (tid < MN) p.partials[(size_t)chunk * MN + tid] = cacc[tid];
  __threadfence();
  __syncthreads();
  __shared__ int s_last;
  const int ngroups = (nchunks + GROUP - 1) / GROUP, grp = chunk / GROUP;
  const int gsize = min(GROUP, nchunks - grp * GROUP);
  if (tid == 0) s_last = (atomicAdd(p.counter + grp, 1u) == (unsigned)(gsize - 1));
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double* Gs = p.partials + (size_t)nchunks * MN;  // [group][MN]
  for (int e = tid; e < MN; e += THREADS) {
    double v[GROUP];
#pragma unroll
    for (int i = 0; i < GROUP; i++) v[i] = i < gsize ? __ldcg(&p.partials[(size_t)(grp * GROUP + i) * MN + e]) : 0.0;
    double sum = 0.0;
#pragma unroll
    for (int i = 0; i < GROUP; i++) sum += v[i];
    Gs[(size_t)grp * MN + e] = sum;
  }
  __threadfence();
  __syncthreads();
  if (tid == 0) {
    p.counter[grp] = 0u;
    s_last = (atomicAdd(p.counter + MAXGROUPS, 1u) == (unsigned)(ngroups - 1));
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  if (tid < MN) {
    double v[MAXGROUPS];
#pragma unroll
    for (int i = 0; i < MAXGROUPS; i++) v[i] = i < ngroups ? __ldcg(&Gs[(size_t)i * MN + tid]) : 0.0;
    double sum = 0.0;
#pragma unroll
    for (int i = 0; i < MAXGROUPS; i++) sum += v[i];
    const int mm = tid % M, nn = tid / M;
    const int64_t ci = (int64_t)nn * p.ldc + mm;
    if (p.out_f32) {  // the one rounding of an FP32 result
      float* c = static_cast<float*>(p.C) + ci;
      *c = (float)(p.beta_zero ? p.alpha * sum : (double)(*c) * p.beta + sum * p.alpha);
    } else {
      double* c = static_cast<double*>(p.C) + ci;
      *c = p.beta_zero ? p.alpha * sum : (*c) * p.beta + sum * p.alpha;
    }
  }
  if (tid == 0) p.counter[MAXGROUPS] = 0u;
}

template <int NP, typename TI>
static skinny_status launch(const Args& a, int grid, int smem, cudaStream_t st) {
  static SmemAttr attr;
  auto kern = split_tsmttsm_kernel<NP, TI>;
  ensure_smem_attr(kern, smem, attr);
  kern<<<grid, THREADS, smem, st>>>(a);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("split tsmttsm launch: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  return SKINNY_OK;
}

}  // namespace split

skinny_status split_product(skinny_handle h, bool tsmm, int64_t M, int64_t N, int64_t K,
                            const double* A, int64_t lda, const void* alpha, const double* B,
                            int64_t ldb, const void* beta, double* C, int64_t ldc,
                            cudaStream_t st, bool autoselect) {
  if (tsmm) return split_tsmm(h, false, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, autoselect);
  return split_tsmttsm_t(h, false, false, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, autoselect);
}

skinny_status split_tsmttsm_t(skinny_handle h, bool in_f32, bool out_f32, int64_t M, int64_t N, int64_t K,
                              const void* A, int64_t lda, const void* alpha, const void* B, int64_t ldb,
                              const void* beta, void* C, int64_t ldc, cudaStream_t st, bool autoselect) {
  using namespace split;
  const int64_t es = in_f32 ? 4 : 8;
  if (M > 128 || N > 128) {
    set_error("split precision TSMTTSM: M, N <= 128");
    return SKINNY_UNSUPPORTED;
  }
  // auto selection (measured on GB300): the split kernel wins from M*N >= 256 on, and whenever
  // both widths are at least 8 (8x8 1.07x at 512 MB of operands and 1.29x at K = 2^20, 8x16 1.37x,
  // 16x8 1.44x; complex 4x8 and 8x4 through the real product 1.3x); below that the CUDA-core FP64
  // kernel is as fast or faster (4x16 0.71x, 4x32 0.44x).  The wide kernel costs about as much per 64 x 64
  // block whatever the block's fill (12.5 ms per block at K = 2^24; CUDA-core FP64 takes 23 ms at
  // M = N = 17 and 114 ms at 64), so it is chosen from M*N >= 320 per block on; with M, N <= 32 its
  // folded stages halve that cost, and with both widths >= 8 it wins from the smallest such
  // product on (1 GiB of operands: 17x8 1.9x, 20x8 1.9x, 17x17 4.8x, 32x8 1.8x; 32x4 is a tie and
  // takes the CUDA-core kernel through the rule above).  The autotuner can override per shape.
  const bool wide = M > 16 || N > 16;
  const int64_t sym_w = (A == B && lda == ldb && M == N) ? 1 : 0;
  const int64_t bm = (M + 63) / 64, bn = (N + 63) / 64;
  const int64_t nblk_w = sym_w ? bm * (bm + 1) / 2 : bm * bn;
  const int64_t per_blk = (M <= 32 && N <= 32) ? 128 : 320;
  const bool narrow_wins = M * N >= 256 || (M >= 8 && N >= 8);
  if (autoselect && (K < 4096 || !narrow_wins || (wide && M * N < per_blk * nblk_w))) {
    set_error("split precision: not selected automatically for this shape");
    return SKINNY_UNSUPPORTED;
  }
  // M or N > 16: the wide kernel (64 x 64 blocks, FP16 digit planes, level accumulators)
  if (wide) return split_wide_t(h, in_f32, out_f32, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st);
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
  a.gram = (A == B) && (lda == ldb) && (M == N);
  const int NP = pow2ceil(a.gram ? M : N);
  a.MP = a.gram ? NP : pow2ceil(M);
  a.NP = NP;
  // rows per round: 128 * R with R the largest power of two whose slicing units (one column and
  // 8 rows each) fit two per slicer thread and whose FP64 and digit stages fit in shared memory
  // (at least two of each; bulk copies of whole rounds where aligned dense rows fit, else the
  // slicers read global memory).  A round's fixed costs -- the slicers' barrier, the hand-offs,
  // the MMA commit -- then spread over as many rows as possible.
  const int cols = a.MP + (a.gram ? 0 : NP);
  a.nmma = std::max(16, 8 * NP);
  a.tmem_cols = std::max(32, 2 * a.nmma);
  a.lbo_a = (uint32_t)(8 * a.MP * 16);
  a.lbo_b = (uint32_t)(a.nmma * 16);
  // a round starts at a multiple of 128 rows, so its bytes start 16-byte aligned with the operand
  const bool aligned = ((uintptr_t)A % 16 == 0) && (a.gram || (uintptr_t)B % 16 == 0);
  const bool dense = lda <= 2 * M + 16 && (a.gram || ldb <= 2 * N + 16);
  const int64_t fixed = HDR + SBYTES + CBYTES + STATIC_RESERVE;
  int64_t dstage = 0;
  a.stages = 0;
  for (int R = PERIOD / 128; R >= 1 && a.stages == 0; R /= 2) {
    if (R * 16 * cols > 2 * SLICERS) continue;
    a.rr = 128 * R;
    const int64_t octs = a.rr / 8;
    a.dig_a = (uint32_t)round_up(octs * a.lbo_a + DPAD, 1024);
    a.dig_b = a.gram ? 0u : (uint32_t)round_up(octs * a.lbo_b, 1024);
    a.tile_a = (uint32_t)round_up((int64_t)a.rr * lda * es, 128);
    const int64_t tile_b = a.gram ? 0 : round_up((int64_t)a.rr * ldb * es, 128);
    dstage = (int64_t)a.dig_a + a.dig_b;
    for (int bulk = (aligned && dense && K > a.rr) ? 1 : 0; bulk >= 0 && a.stages == 0; bulk--) {
      a.bulk = bulk;
      a.stage_bytes = bulk ? (uint32_t)round_up(a.tile_a + tile_b, 1024) : 1024u;
      for (int dst = MAXDST; dst >= 2 && a.stages == 0; dst--)
        for (int nst = MAXST; nst >= 2; nst--)
          if (fixed + (int64_t)nst * a.stage_bytes + (int64_t)dst * dstage <= h->dev.smem_optin) {
            a.stages = nst;
            a.dstages = dst;
            break;
          }
    }
  }
  if (a.stages == 0) {
    set_error("split precision: stages do not fit in shared memory");
    return SKINNY_UNSUPPORTED;
  }
  a.nrounds = (K + a.rr - 1) / a.rr;
  const int smem2 =
      (int)(fixed - STATIC_RESERVE + (int64_t)a.stages * a.stage_bytes + (int64_t)a.dstages * dstage);
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>({a.nrounds, h->dev.sms, (int64_t)GROUP * MAXGROUPS}));
  Workspace& ws = h->ws[st];
  // CTA partials, then the group sums
  skinny_status s = workspace_ensure(ws, ((size_t)grid + MAXGROUPS) * M * N * 8, st);
  if (s != SKINNY_OK) return s;
  a.partials = (double*)ws.partials;
  a.counter = ws.counter;
  a.err = h->err;
  if (!in_f32) {
    switch (NP) {
      case 1: return launch<1, double>(a, (int)grid, smem2, st);
      case 2: return launch<2, double>(a, (int)grid, smem2, st);
      case 4: return launch<4, double>(a, (int)grid, smem2, st);
      case 8: return launch<8, double>(a, (int)grid, smem2, st);
      case 16: return launch<16, double>(a, (int)grid, smem2, st);
    }
  } else {
    switch (NP) {
      case 1: return launch<1, float>(a, (int)grid, smem2, st);
      case 2: return launch<2, float>(a, (int)grid, smem2, st);
      case 4: return launch<4, float>(a, (int)grid, smem2, st);
      case 8: return launch<8, float>(a, (int)grid, smem2, st);
      case 16: return launch<16, float>(a, (int)grid, smem2, st);
    }
  }
  set_error("split precision: unsupported N");
  return SKINNY_UNSUPPORTED;
}

}  // namespace skinny
