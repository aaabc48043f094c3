// split.cu -- FP64 TSMTTSM in split precision on tcgen05 tensor cores for M, N <= 16 (no
// counterpart in the reference, whose FP64 kernels are CUDA-core DFMA loops, e.g.
// tsmttsm/genv5.cuh:28-89).  Wider products go to split_wide.cu.
//
// Why: GB300 executes 595 G FP64 FMA/s but 2.25 P FP16 / BF16 tensor flop/s.  A CUDA-core FP64 TSMTTSM
// is FP64-bound for every M = N >= 2.  Here each FP64 product is computed exactly from 8-bit
// pieces on the tensor cores, and FP64 arithmetic is used only a few times per 1024 rows.
//
// Scheme (Ozaki-style error-free splitting, written for this kernel):
//   * Per column m of A (and n of B) a shared exponent E is kept: the largest exponent field
//     seen in the current accumulation period.  Each element x is written as a 62-bit fixed-point
//     integer F = |x| * 2^(1084 - E) (< 2^62) and F as 8 balanced base-256 digits
//     d_1..d_8 in [-128, 128] (d_1 most significant): x = sign * sum_i d_i 2^(8(8-i)) 2^(E-1084).
//     Digits are exact in FP16 (formed with byte permutes, digits.cuh).
//   * Digit planes are stacked along the MMA dimensions: A rows (i-1)*MP + m, B rows
//     (j-1)*NP + n, so one tcgen05.mma (M = 128, N = 8*NP, K = 16, FP16 x FP16 -> FP32 in TMEM)
//     forms every digit-pair product d_i(a) d_j(b) for 16 rows of K.
//   * |d_i d_j| <= 2^14, so over a period of <= 1024 rows every partial sum is an integer of
//     magnitude <= 2^24: the FP32 accumulation in TMEM is exact.  A period ends after 1024 rows,
//     or earlier when a window raises a column's exponent.
//   * Drain: TMEM -> registers -> int32; level sums S_L = sum_{i+j=L} D_ij (L = 2..9) are formed
//     with a per-lane rotation and warp shuffles, then in shared memory with integer atomics;
//     V = sum_L S_L 2^(8(16-L)) is assembled from two int64 words and added to an FP64 accumulator
//     per C entry with weight 2^(EA+EB-2168).  Levels L >= 10 are dropped: their weight is below
//     2^-56 of the leading level.
//   * K rows stream in windows of 128 rows through a ring of FP64 tiles (1-D TMA bulk copies);
//     digit buffers are double-buffered so slicing window w+1 overlaps the MMAs of window w.
//   * Cross-CTA finish as in the CUDA-core kernel: CTA partials in FP64, the last CTA (ticket)
//     sums them in CTA order, applies alpha/beta.
// Inputs must be finite (Inf/NaN have no fixed-point form).

#include <cstring>

#include "api_internal.h"
#include "digits.cuh"

namespace skinny {

namespace split {

constexpr int W = 128;          // rows per window (8 MMA K-steps of 16)
constexpr int PERIOD = 1024;    // rows accumulated exactly in TMEM
constexpr int THREADS = 256;
constexpr int DIGITS = 8;
constexpr int OCT = W / 8;      // k-octets per window
constexpr int DPAD = 128 * 16;  // slack after an A digit buffer: the MMA reads 128 rows per k-octet
constexpr int HDR = 1024;       // barriers, TMEM slot, exponents
constexpr int SBYTES = 8 * 16 * 16 * 4;  // level sums S[8][16][16]

struct Args {
  const double* A;
  const double* B;
  double* C;
  int64_t K, lda, ldb, ldc;
  int M, N, MP;
  double alpha, beta;
  int beta_zero, gram, bulk, stages;
  int64_t ntiles;
  uint32_t tile_a, tile_b;  // bytes per FP64 stage (A, B), multiples of 128
  int64_t lda_s, ldb_s;     // row strides of the FP64 stage tiles
  int nmma;                 // MMA N (multiple of 16, >= 16)
  int tmem_cols;
  int sw;                   // windows per super-window (rows per iteration = sw * W)
  uint32_t lbo_a, lbo_b;    // bytes between k-octets of the A / B digit buffers
  uint32_t dig_a, dig_b;    // bytes of one A / B digit buffer (A includes DPAD)
  double* partials;
  unsigned* counter;
  int* err;
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

template <int NP>
__global__ void __launch_bounds__(THREADS, 1) split_tsmttsm_kernel(const Args p) {
  const int chunk = blockIdx.x, nchunks = gridDim.x;
  constexpr int BN = NP < 8 ? NP : 8;  // n per drain block
  constexpr int NB = NP / BN;          // drain blocks
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* bar_tma = reinterpret_cast<uint64_t*>(smem);       // [4]
  uint64_t* bar_mma = reinterpret_cast<uint64_t*>(smem + 32);  // [2]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem + 64);
  int* EAc = reinterpret_cast<int*>(smem + 128);
  int* EBc = EAc + 16;
  int* EAw = EAc + 32;
  int* EBw = EAc + 48;
  int* S = reinterpret_cast<int*>(smem + HDR);
  unsigned char* ring = smem + HDR + SBYTES;
  const uint32_t stage_bytes = p.tile_a + p.tile_b;
  unsigned char* dig = ring + (size_t)p.stages * stage_bytes;  // 1024-aligned by the host
  auto digA = [&](int b) { return dig + (size_t)b * (p.dig_a + p.dig_b); };
  auto digB = [&](int b) { return p.gram ? digA(b) : digA(b) + p.dig_a; };
  auto tileA = [&](int s) { return reinterpret_cast<double*>(ring + (size_t)s * stage_bytes); };
  auto tileB = [&](int s) {
    return p.gram ? tileA(s) : reinterpret_cast<double*>(ring + (size_t)s * stage_bytes + p.tile_a);
  };

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int M = p.M, N = p.N, MP = p.gram ? NP : p.MP;
  const int RSW = p.sw * W;  // rows per super-window
  const int64_t t_begin = p.ntiles * chunk / nchunks;
  const int64_t t_end = p.ntiles * (chunk + 1) / nchunks;
  const int nt = (int)(t_end - t_begin);
  auto is_bulk = [&](int64_t t) { return p.bulk && (t + 1) * (int64_t)RSW < p.K; };
  auto issue = [&](int64_t t, int s) {
    const int64_t r0 = t * RSW;
    const uint32_t ba = (uint32_t)(RSW * p.lda * 8), bb = p.gram ? 0u : (uint32_t)(RSW * p.ldb * 8);
    mbar_arrive_expect_tx(&bar_tma[s], ba + bb);
    bulk_g2s(tileA(s), p.A + r0 * p.lda, ba, &bar_tma[s]);
    if (!p.gram) bulk_g2s(tileB(s), p.B + r0 * p.ldb, bb, &bar_tma[s]);
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
  if (tid < 64) EAc[tid] = 0;  // EAc, EBc, EAw, EBw
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  if (p.bulk && tid == 0)
    for (int i = 0; i < nt && i < p.stages; i++)
      if (is_bulk(t_begin + i)) issue(t_begin + i, i);

  // idesc: D f32, A/B f16, K-major both, N = nmma, M = 128
  const uint32_t idesc = (1u << 4) | ((uint32_t)(p.nmma >> 3) << 17) | ((128u >> 4) << 24);

  // Slicing units: (operand, column c, k-octet o).  A units u < nA: c = u % MP, o = u / MP;
  // B units nA <= u < nA + nB: c = (u - nA) % NP.  nA is a multiple of 32, so a warp holds units
  // of one operand and lanes with equal c sit at xor distances that are multiples of MP (NP).
  const int nA = p.sw * OCT * MP;
  const int nA_al = (nA + 31) & ~31;  // B units start on a warp boundary
  const int nB = p.gram ? 0 : p.sw * OCT * NP;
  const int nU = nA_al + nB;          // <= 2 * THREADS (host guarantees)
  const int u0 = tid, u1 = tid + THREADS;
  double cacc = 0.0;  // FP64 accumulator of C entry tid (tid < M*N), CTA-local
  int uses[2] = {0, 0};
  int period_rows = 0;
  bool active = false;
  bool bail = false;

  // ---- drain: TMEM -> level sums -> FP64 accumulators -------------------------------------------
  auto drain = [&]() {
    for (int e = tid; e < 8 * 16 * 16; e += THREADS) S[e] = 0;
    __syncthreads();
    tc_fence_after();
    const int q = warp & 3, half = warp >> 2;
    const int r = 32 * q + lane;  // TMEM lane = A digit row
    const int i0 = r / MP, m = r - i0 * MP;  // digit index (0-based) and column of A
    const bool rvalid = (i0 < DIGITS) && (m < M);
    for (int nb = half; nb < NB; nb += 2) {
      uint32_t raw[DIGITS][BN];
#pragma unroll
      for (int j = 0; j < DIGITS; j++) {
        uint32_t tmp[BN];
        tmem_ld<BN>(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(j * NP + nb * BN), tmp);
#pragma unroll
        for (int x = 0; x < BN; x++) raw[j][x] = tmp[x];
      }
      tmem_wait_ld();
#pragma unroll
      for (int x = 0; x < BN; x++) {
        const int n = nb * BN + x;
        int R[DIGITS];
#pragma unroll
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
#pragma unroll
        for (int t = 0; t < DIGITS; t++) {
          int c = (i0 <= t) ? R[t] : 0;
          for (int o = MP; o < 32; o <<= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
          if (lane < MP && rvalid && n < N) atomicAdd(&S[(t * 16 + m) * 16 + n], c);
        }
      }
    }
    tc_fence_before();
    __syncthreads();
    if (tid < M * N) {
      const int mm = tid % M, nn = tid / M;
      long long s[8];
#pragma unroll
      for (int t = 0; t < 8; t++) s[t] = S[(t * 16 + mm) * 16 + nn];
      const long long vhi = (s[0] << 24) + (s[1] << 16) + (s[2] << 8) + s[3];
      const long long vlo = (s[4] << 24) + (s[5] << 16) + (s[6] << 8) + s[7];
      const int ea = EAc[mm], eb = p.gram ? EAc[nn] : EBc[nn];
      const double v = fma((double)vlo, 0x1p-32, (double)vhi);  // in units of 2^(EA+EB-2080)
      cacc = fma(v * pow2i(ea - 1040), pow2i(eb - 1040), cacc);
    }
  };

  auto unit_info = [&](int u, bool& isA, int& c, int& o, bool& valid) {
    isA = u < nA_al;
    const int v = isA ? u : u - nA_al;
    const int CP = isA ? MP : NP;
    c = v % CP;
    o = v / CP;
    valid = (isA ? v < nA : v < nB) && c < (isA ? M : N);
  };

  for (int it = 0; it < nt && !bail; it++) {
    const int64_t t = t_begin + it;
    const int s = it % p.stages;
    const int64_t r0 = t * RSW;
    const int rows = (int)((p.K - r0) < RSW ? (p.K - r0) : RSW);
    double* TA = tileA(s);
    double* TB = tileB(s);
    if (is_bulk(t)) {
      bool ok = mbar_wait_bounded(&bar_tma[s], (uint32_t)((it / p.stages) & 1), p.err);
      if (__syncthreads_or(!ok)) {
        bail = true;
        break;
      }
    } else {
      for (int e = tid; e < rows * M; e += THREADS) {
        int rr = e / M, c = e - rr * M;
        TA[rr * p.lda_s + c] = p.A[(r0 + rr) * p.lda + c];
      }
      if (!p.gram)
        for (int e = tid; e < rows * N; e += THREADS) {
          int rr = e / N, c = e - rr * N;
          TB[rr * p.ldb_s + c] = p.B[(r0 + rr) * p.ldb + c];
        }
      __syncthreads();
    }
    // load my (up to two) units and reduce the super-window's exponent maxima
    double v[2][8];
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int u = k ? u1 : u0;
      bool isA, valid;
      int c, o;
      unit_info(u, isA, c, o, valid);
      const double* T = isA ? TA : TB;
      const int64_t ld = isA ? p.lda_s : p.ldb_s;
      uint32_t e = 0;
#pragma unroll
      for (int q2 = 0; q2 < 8; q2++) {
        const int rr = o * 8 + q2;
        v[k][q2] = (valid && rr < rows) ? T[rr * ld + c] : 0.0;
        e = max(e, exp_field(v[k][q2]));
      }
      if (u - lane < nU) {  // warp-uniform: the warp holds units
        const int CP = isA ? MP : NP;
        for (int x = CP; x < 32; x <<= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, x));
        if (lane < CP && valid && e) atomicMax(isA ? &EAw[c] : &EBw[c], (int)e);
      }
    }
    __syncthreads();
    bool need = !active || period_rows + RSW > PERIOD;
    if (tid < M && EAw[tid] > EAc[tid]) need = true;
    if (!p.gram && tid < N && EBw[tid] > EBc[tid]) need = true;
    if (__syncthreads_or(need)) {
      if (active) {
        const int bl = (it - 1) & 1;
        bool ok = mbar_wait_bounded(&bar_mma[bl], (uint32_t)((uses[bl] - 1) & 1), p.err);
        if (__syncthreads_or(!ok)) {
          bail = true;
          break;
        }
        drain();
      }
      __syncthreads();
      if (tid < M) EAc[tid] = max(EAc[tid], EAw[tid]);
      if (!p.gram && tid < N) EBc[tid] = max(EBc[tid], EBw[tid]);
      period_rows = 0;
      __syncthreads();
    }
    const int b = it & 1;
    if (uses[b] > 0) {
      bool ok = mbar_wait_bounded(&bar_mma[b], (uint32_t)((uses[b] - 1) & 1), p.err);
      if (__syncthreads_or(!ok)) {
        bail = true;
        break;
      }
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int u = k ? u1 : u0;
      bool isA, valid;
      int c, o;
      unit_info(u, isA, c, o, valid);
      if (valid) {
        if (isA)
          slice_unit(v[k], (uint32_t)EAc[c], c, MP, o, p.lbo_a, digA(b));
        else
          slice_unit(v[k], (uint32_t)EBc[c], c, NP, o, p.lbo_b, digB(b));
      }
    }
    if (tid < 16) EAw[tid] = 0;
    else if (tid < 32) EBw[tid - 16] = 0;
    fence_proxy_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(digA(b)), b0 = smem_u32(digB(b));
      const uint32_t lbb = p.gram ? p.lbo_a : p.lbo_b;
      const int ksteps = RSW / 16;
      for (int ks = 0; ks < ksteps; ks++)
        mma_f16(tmem, make_desc(a0 + 2 * ks * p.lbo_a, p.lbo_a), make_desc(b0 + 2 * ks * lbb, lbb), idesc,
                 (period_rows > 0 || ks > 0) ? 1u : 0u);
      mma_commit(&bar_mma[b]);
      if (p.bulk && it + p.stages < nt && is_bulk(t + p.stages)) {
        fence_proxy_async_smem();
        issue(t + p.stages, s);
      }
    }
    uses[b]++;
    period_rows += RSW;
    active = true;
  }

  if (!bail && active) {
    const int bl = (nt - 1) & 1;
    bool ok = mbar_wait_bounded(&bar_mma[bl], (uint32_t)((uses[bl] - 1) & 1), p.err);
    if (__syncthreads_or(!ok))
      bail = true;
    else
      drain();
  }
  if (bail) {
    // let MMAs already issued finish before the TMEM is released (bounded)
    for (int bb = 0; bb < 2; bb++)
      if (uses[bb] > 0) mbar_wait_bounded(&bar_mma[bb], (uint32_t)((uses[bb] - 1) & 1), nullptr);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(p.tmem_cols));
  if (bail) return;

  // ---- cross-CTA finish -----------------------------------------------------------------------
  const int MN = M * N;
  if (tid < MN) p.partials[(size_t)chunk * MN + tid] = cacc;
  __threadfence();
  __syncthreads();
  __shared__ int s_last;
  if (tid == 0) s_last = (atomicAdd(p.counter, 1u) == (unsigned)(nchunks - 1));
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double* red = reinterpret_cast<double*>(ring);
  const int P = THREADS / MN;  // >= 1 since MN <= 256
  const int e = tid % MN, j = tid / MN;
  const int nb = nchunks;
  if (j < P) {
    double sum = 0.0;
    const int b0 = (int)((int64_t)nb * j / P), b1 = (int)((int64_t)nb * (j + 1) / P);
    for (int bb = b0; bb < b1; bb++) sum += __ldcg(&p.partials[(size_t)bb * MN + e]);
    red[j * MN + e] = sum;
  }
  __syncthreads();
  if (tid < MN) {
    double sum = red[tid];
    for (int q2 = 1; q2 < P; q2++) sum += red[q2 * MN + tid];
    const int mm = tid % M, nn = tid / M;
    double* c = p.C + (int64_t)nn * p.ldc + mm;
    *c = p.beta_zero ? p.alpha * sum : (*c) * p.beta + sum * p.alpha;
  }
  if (tid == 0) *p.counter = 0u;
}

template <int NP>
static skinny_status launch(const Args& a, int grid, int smem, cudaStream_t st) {
  static SmemAttr attr;
  auto kern = split_tsmttsm_kernel<NP>;
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
  using namespace split;
  if (tsmm) return split_tsmm(h, false, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, autoselect);
  if (M > 128 || N > 128) {
    set_error("split precision TSMTTSM: M, N <= 128");
    return SKINNY_UNSUPPORTED;
  }
  // auto selection (measured on GB300): the split kernel wins from M*N >= 256 on, and whenever
  // both widths are at least 8 (8x8 1.07x at 512 MB of operands and 1.29x at K = 2^20, 8x16 1.37x,
  // 16x8 1.44x; complex 4x8 and 8x4 through the real product 1.3x); below that the CUDA-core FP64
  // kernel is as fast or faster (4x16 0.71x, 4x32 0.44x).  The wide kernel costs about as much per 64 x 64
  // block whatever the block's fill (12.5 ms per block at K = 2^24; CUDA-core FP64 takes 23 ms at
  // M = N = 17 and 114 ms at 64), so it is chosen from M*N >= 320 per block on.  The autotuner can
  // override per shape.
  const bool wide = M > 16 || N > 16;
  const int64_t sym_w = (A == B && lda == ldb && M == N) ? 1 : 0;
  const int64_t bm = (M + 63) / 64, bn = (N + 63) / 64;
  const int64_t nblk_w = sym_w ? bm * (bm + 1) / 2 : bm * bn;
  const bool narrow_wins = M * N >= 256 || (M >= 8 && N >= 8);
  if (autoselect && (K < 4096 || !narrow_wins || (wide && M * N < 320 * nblk_w))) {
    set_error("split precision: not selected automatically for this shape");
    return SKINNY_UNSUPPORTED;
  }
  // M or N > 16: the wide kernel (64 x 64 blocks, FP16 digit planes, level accumulators)
  if (wide) return split_wide(h, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st);
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
  std::memcpy(&a.alpha, alpha, 8);
  std::memcpy(&a.beta, beta, 8);
  a.beta_zero = a.beta == 0.0;
  a.gram = (A == B) && (lda == ldb) && (M == N);
  const int NP = pow2ceil(a.gram ? M : N);
  a.MP = a.gram ? NP : pow2ceil(M);
  // windows per iteration: the largest power of two (<= PERIOD / W) whose slicing units
  // (k-octet x column; A units padded to a warp multiple) fit two per thread
  auto units = [&](int w) {
    return (int)round_up((int64_t)w * OCT * a.MP, 32) + (a.gram ? 0 : w * OCT * NP);
  };
  int sw = PERIOD / W;
  while (sw > 1 && units(sw) > 2 * THREADS) sw >>= 1;
  if (units(sw) > 2 * THREADS) {
    set_error("split precision: too many slicing units");
    return SKINNY_UNSUPPORTED;
  }
  a.sw = sw;
  const int64_t RSW = (int64_t)sw * W;
  const bool aligned = ((uintptr_t)A % 16 == 0) && (a.gram || (uintptr_t)B % 16 == 0);
  const bool dense = lda <= 2 * M + 16 && (a.gram || ldb <= 2 * N + 16);
  a.nmma = std::max(16, 8 * NP);
  a.tmem_cols = a.nmma <= 32 ? 32 : (a.nmma <= 64 ? 64 : 128);
  a.lbo_a = (uint32_t)(8 * a.MP * 16);
  a.lbo_b = (uint32_t)(a.nmma * 16);
  const int64_t octs = (int64_t)sw * OCT;
  a.dig_a = (uint32_t)round_up(octs * a.lbo_a + DPAD, 1024);
  a.dig_b = a.gram ? 0u : (uint32_t)round_up(octs * a.lbo_b, 1024);
  const int64_t dig = (int64_t)2 * (a.dig_a + a.dig_b);
  const int64_t fixed = HDR + SBYTES + dig;
  // FP64 stages: whole (padded) rows by bulk copy where they fit two stages, else the M (N) used
  // columns by plain loads
  int64_t stage = 0;
  int stages = 0;
  for (int bulk = (aligned && dense && K > RSW) ? 1 : 0; bulk >= 0; bulk--) {
    a.bulk = bulk;
    a.lda_s = a.bulk ? lda : M;
    a.ldb_s = a.gram ? a.lda_s : (a.bulk ? ldb : N);
    a.tile_a = (uint32_t)round_up(RSW * a.lda_s * 8, 128);
    a.tile_b = a.gram ? 0u : (uint32_t)round_up(RSW * a.ldb_s * 8, 128);
    stage = round_up(a.tile_a + a.tile_b, 1024);
    stages = (int)std::min<int64_t>(4, (h->dev.smem_optin - fixed) / stage);
    if (stages >= 2) break;
  }
  if (a.gram)
    a.tile_a = (uint32_t)stage;
  else
    a.tile_b = (uint32_t)(stage - a.tile_a);
  if (stages < 2) {
    set_error("split precision: tiles do not fit in shared memory");
    return SKINNY_UNSUPPORTED;
  }
  a.stages = stages;
  a.ntiles = (K + RSW - 1) / RSW;
  const int smem2 = (int)(fixed + stages * stage);
  const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(a.ntiles, h->dev.sms));
  Workspace& ws = h->ws[st];
  skinny_status s = workspace_ensure(ws, (size_t)grid * M * N * 8, st);
  if (s != SKINNY_OK) return s;
  a.partials = (double*)ws.partials;
  a.counter = ws.counter;
  a.err = h->err;
  switch (NP) {
    case 1: return launch<1>(a, (int)grid, smem2, st);
    case 2: return launch<2>(a, (int)grid, smem2, st);
    case 4: return launch<4>(a, (int)grid, smem2, st);
    case 8: return launch<8>(a, (int)grid, smem2, st);
    case 16: return launch<16>(a, (int)grid, smem2, st);
  }
  set_error("split precision: unsupported N");
  return SKINNY_UNSUPPORTED;
}

}  // namespace skinny
