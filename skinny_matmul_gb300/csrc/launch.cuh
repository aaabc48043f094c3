// launch.cuh -- host-side planning and launch of the CUDA-core TSMTTSM / TSMM kernels.
//
// The reference fixes (M, N) at compile time and picks one variant per binary
// (Makefile:11-20, versions.hpp:48-177, tsmm/fix_blend.cuh:7-29).  Here (M, N) are runtime
// values: the plan picks a register tile (TM x TN) per thread from a small set of compiled
// shapes, a row-tile size for the shared-memory ring, the ring depth and a persistent grid of
// one wave.  An autotuned grid size (blocks per SM) may override the default.
#pragma once
#include <algorithm>
#include <atomic>
#include <string>

#include "skinny.h"
#include "tsmm.cuh"
#include "tsmttsm.cuh"
#include "tsmttsm_rows.cuh"

namespace skinny {

struct DeviceInfo {
  int id = 0;
  int sms = 0;
  int smem_optin = 0;
  uint32_t wait_polls = kWaitPolls;  // poll limit of the CUDA-core TSMTTSM's bounded waits
};

// Per-(handle, stream) workspace: CTA partials + ticket counter for the in-launch reduction.
struct Workspace {
  void* partials = nullptr;
  size_t bytes = 0;
  unsigned* counter = nullptr;
};

// Implemented in api.cu: grow the workspace to `bytes` (synchronises `stream` before freeing
// the old buffer) and make sure the ticket counter exists and is zero.
skinny_status workspace_ensure(Workspace& ws, size_t bytes, cudaStream_t stream);
void set_error(const std::string& msg);
// Counts every kernel launch of the library (skinny_kernel_launches()).
void count_launch();

// Launch options chosen by the caller (autotuner / request loop).  0 = default.
struct LaunchOpts {
  int blocks_per_sm = 0;
  int rows_per_tile = 0;
  int method = -1;  // for SKINNY_ACC_AUTO: the method the autotuner measured fastest (-1: none)
};

inline int pow2ceil(int64_t v) {
  int p = 1;
  while (p < v && p < (1 << 30)) p <<= 1;
  return p;
}
inline int64_t round_up(int64_t v, int64_t m) { return (v + m - 1) / m * m; }

// The dynamic shared-memory attribute a kernel has been given, per device (the attribute is set
// per device: cudaFuncSetAttribute acts on the current one).  Zero-initialised as a static.
constexpr int kMaxDevices = 64;
struct SmemAttr {
  std::atomic<int> bytes[kMaxDevices];
};

// Raises `kernel`'s dynamic shared-memory limit on the current device to at least `bytes`;
// records only a successful call.  Returns false if the attribute could not be set.
template <typename K>
inline bool ensure_smem_attr(K kernel, int bytes, SmemAttr& done) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) == cudaSuccess;
  }
  std::atomic<int>& d = done.bytes[dev];
  if (d.load(std::memory_order_relaxed) >= bytes) return true;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) {
    cudaGetLastError();
    set_error("cudaFuncSetAttribute(MaxDynamicSharedMemorySize) failed");
    return false;
  }
  int cur = d.load();
  while (cur < bytes && !d.compare_exchange_weak(cur, bytes)) {
  }
  return true;
}

// ----------------------------------------------------------------------------------- TSMTTSM
template <typename T, typename Acc, int TM, int TN>
skinny_status tsmttsm_launch_tile(const TsmttsmArgs<T>& a, dim3 grid, int smem, cudaStream_t st) {
  static SmemAttr attr;
  auto kern = tsmttsm_kernel<T, Acc, TM, TN>;
  ensure_smem_attr(kern, smem, attr);
  kern<<<grid, TSMTTSM_THREADS, smem, st>>>(a);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("tsmttsm launch: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  return SKINNY_OK;
}

// Register-tile entries (accumulators) a thread of the ring kernel may hold: 64 FP64-sized ones,
// 32 of 16 bytes, 8 of 32 bytes (complex double-double)
template <typename Acc>
constexpr int tile_cap() {
  return sizeof(Acc) >= 32 ? 8 : (int)(128 / (sizeof(Acc) / 4));
}

template <typename T, typename Acc>
skinny_status tsmttsm_dispatch(int tm, int tn, const TsmttsmArgs<T>& a, dim3 grid, int smem,
                               cudaStream_t st) {
#define SK_TILE(X, Y)                                                                   \
  if constexpr (X * Y <= tile_cap<Acc>() && X * Y <= 64)                                \
    if (tm == X && tn == Y) return tsmttsm_launch_tile<T, Acc, X, Y>(a, grid, smem, st);
  SK_TILE(1, 1) SK_TILE(1, 2) SK_TILE(1, 4) SK_TILE(1, 8)
  SK_TILE(2, 1) SK_TILE(2, 2) SK_TILE(2, 4) SK_TILE(2, 8)
  SK_TILE(4, 1) SK_TILE(4, 2) SK_TILE(4, 4) SK_TILE(4, 8)
  SK_TILE(8, 1) SK_TILE(8, 2) SK_TILE(8, 4) SK_TILE(8, 8)
#undef SK_TILE
  set_error("tsmttsm: no compiled register tile");
  return SKINNY_UNSUPPORTED;
}

struct TsmttsmPlan {
  int tm, tn, rows, stages, grid, groups, smem, bulk;
  int64_t ntiles, lda_s, ldb_s;
  size_t partial_bytes;
};

template <typename T, typename Acc>
skinny_status tsmttsm_plan(const DeviceInfo& dev, int64_t M, int64_t N, int64_t K, const void* A,
                           int64_t lda, const void* B, int64_t ldb, bool gram, const LaunchOpts& o,
                           TsmttsmPlan& pl) {
  const int cap = tile_cap<Acc>();
  int tm = pow2ceil(M) < 8 ? pow2ceil(M) : 8;
  int tn = pow2ceil(N) < 8 ? pow2ceil(N) : 8;
  while (tm * tn > cap) (tm >= tn ? tm : tn) /= 2;
  const int64_t Gall = ((M + tm - 1) / tm) * ((N + tn - 1) / tn);
  const int64_t groups = (Gall + TSMTTSM_THREADS - 1) / TSMTTSM_THREADS;
  if (groups > 64) {  // one ticket counter per group in the 256-byte counter block
    set_error("tsmttsm: M, N too large for the CUDA-core kernel");
    return SKINNY_UNSUPPORTED;
  }
  const int64_t G = Gall < TSMTTSM_THREADS ? Gall : TSMTTSM_THREADS;
  const int RS = (int)(TSMTTSM_THREADS / G);
  const int64_t s = sizeof(T);
  const bool aligned = ((uintptr_t)A % 16 == 0) && (gram || (uintptr_t)B % 16 == 0);
  const bool dense = lda <= 2 * M + 16 && (gram || ldb <= 2 * N + 16);
  // shared row strides: ld when bulk-copied, dense (M / N) when loaded by threads
  int64_t row_bytes_bulk = (lda + (gram ? 0 : ldb)) * s;
  int64_t row_bytes_dense = (M + (gram ? 0 : N)) * s;
  int rows = o.rows_per_tile;
  int64_t rb = (aligned && dense) ? row_bytes_bulk : row_bytes_dense;
  if (rows <= 0) {
    int64_t r = 16384 / rb;
    rows = 16;
    while (rows * 2 <= r && rows < 1024) rows *= 2;
  }
  rows = (int)round_up(rows < RS ? RS : rows, 16);
  const int64_t stage_a = round_up(rows * (aligned && dense ? lda : M) * s, 128);
  const int64_t stage_b = gram ? 0 : round_up(rows * (aligned && dense ? ldb : N) * s, 128);
  const int64_t stage = stage_a + stage_b;
  const bool bulk = aligned && dense && stage <= 65536 && K > rows;
  const int64_t budget = (int64_t)dev.smem_optin - SMEM_HEADER - 1024;
  int stages = (int)std::min<int64_t>(8, (160 * 1024) / std::max<int64_t>(stage, 1));
  if (stages < 2) stages = 2;
  if (stages * stage > budget) stages = (int)(budget / stage);
  if (stages < 1) {
    set_error("tsmttsm: row tile does not fit in shared memory");
    return SKINNY_UNSUPPORTED;
  }
  pl.tm = tm;
  pl.tn = tn;
  pl.rows = rows;
  pl.stages = stages;
  pl.bulk = bulk;
  pl.lda_s = bulk ? lda : M;
  pl.ldb_s = gram ? pl.lda_s : (bulk ? ldb : N);
  pl.ntiles = (K + rows - 1) / rows;
  int64_t smem = SMEM_HEADER + stages * stage;
  const int64_t red = (int64_t)(M * N + TSMTTSM_THREADS) * sizeof(Acc);
  if (red + SMEM_HEADER <= budget && smem < SMEM_HEADER + red) smem = SMEM_HEADER + red;
  pl.smem = (int)smem;
  const int bps = o.blocks_per_sm > 0 ? o.blocks_per_sm : 1;
  int64_t grid = (int64_t)dev.sms * bps;
  if (grid > pl.ntiles) grid = pl.ntiles;
  if (grid < 1) grid = 1;
  pl.grid = (int)grid;
  pl.groups = (int)groups;
  pl.partial_bytes = (size_t)grid * (size_t)(M * N) * sizeof(Acc);
  return SKINNY_OK;
}

// ----------------------------------------------------------------- TSMTTSM, narrow products
// Register-tile entries a thread of the row-streaming kernel may hold: 64 for 4- and 8-byte
// accumulators (FP64 8 x 8), 16 for 16-byte ones (complex FP64, double-double), 4 for 32-byte
// ones (complex double-double).
template <typename Acc>
constexpr int rows_cap() {
  return sizeof(Acc) <= 8 ? 64 : (sizeof(Acc) <= 16 ? 16 : 4);
}

// The row-streaming kernel takes a product when both padded widths are <= 8 and their tile fits
// rows_cap; an autotuned row-tile size asks for the ring kernel instead.
template <typename T, typename Acc>
bool rows_eligible(int64_t M, int64_t N, bool gram, const LaunchOpts& o) {
  if (o.rows_per_tile > 0 || M < 1 || N < 1 || M > 8 || N > 8) return false;
  int tm = pow2ceil(M), tn = pow2ceil(N);
  if (gram) tm = tn = std::max(tm, tn);
  return tm * tn <= rows_cap<Acc>();
}

template <typename T, typename Acc, int TM, int TN>
skinny_status tsmttsm_rows_launch(RowsArgs<T>& a, const DeviceInfo& dev, Workspace& ws, int bps_opt,
                                  cudaStream_t st) {
  if constexpr (TM * TN > rows_cap<Acc>()) {
    set_error("tsmttsm: register tile too large for the accumulator type");
    return SKINNY_UNSUPPORTED;
  } else {
    constexpr int U = TM * TN <= 2 ? 4 : (TM * TN <= 8 ? 2 : 1);
    auto kern = tsmttsm_rows_kernel<T, Acc, TM, TN, U>;
    int occ = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, ROWS_THREADS, 0);
    if (occ < 1) occ = 1;
    if (bps_opt > 0 && bps_opt < occ) occ = bps_opt;
    const int64_t per_cta = (int64_t)ROWS_THREADS * U;
    int64_t grid = std::min<int64_t>((int64_t)dev.sms * occ, (a.K + per_cta - 1) / per_cta);
    if (grid < 1) grid = 1;
    skinny_status s = workspace_ensure(ws, (size_t)grid * (size_t)(a.M * a.N) * sizeof(Acc), st);
    if (s != SKINNY_OK) return s;
    a.partials = ws.partials;
    a.counter = ws.counter;
    kern<<<(int)grid, ROWS_THREADS, 0, st>>>(a);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      set_error(std::string("tsmttsm launch: ") + cudaGetErrorString(e));
      return SKINNY_DEVICE_ERROR;
    }
    return SKINNY_OK;
  }
}

template <typename T, typename Acc>
skinny_status tsmttsm_rows_run(const DeviceInfo& dev, Workspace& ws, cudaStream_t st, int64_t M, int64_t N,
                               int64_t K, const T* A, int64_t lda, T alpha, const T* B, int64_t ldb, T beta,
                               bool beta_zero, T* C, int64_t ldc, bool gram, const LaunchOpts& o) {
  int tm = pow2ceil(M), tn = pow2ceil(N);
  if (gram) tm = tn = std::max(tm, tn);
  RowsArgs<T> a;
  a.A = A;
  a.B = B;
  a.C = C;
  a.K = K;
  a.lda = lda;
  a.ldb = ldb;
  a.ldc = ldc;
  a.M = (int)M;
  a.N = (int)N;
  a.alpha = alpha;
  a.beta = beta;
  a.beta_zero = beta_zero;
  a.gram = gram;
  // 16-byte pairs: FP64, an aligned base, an even leading dimension covering the padded width
  const bool f64 = std::is_same<T, double>::value;
  a.vec_a = f64 && tm >= 2 && (uintptr_t)A % 16 == 0 && lda % 2 == 0 && lda >= tm;
  a.vec_b = f64 && tn >= 2 && (uintptr_t)B % 16 == 0 && ldb % 2 == 0 && ldb >= tn;
  a.partials = nullptr;
  a.counter = nullptr;
  const int b = o.blocks_per_sm;
#define SK_ROWS(X, Y) \
  if (tm == X && tn == Y) return tsmttsm_rows_launch<T, Acc, X, Y>(a, dev, ws, b, st);
  SK_ROWS(1, 1) SK_ROWS(1, 2) SK_ROWS(1, 4) SK_ROWS(1, 8)
  SK_ROWS(2, 1) SK_ROWS(2, 2) SK_ROWS(2, 4) SK_ROWS(2, 8)
  SK_ROWS(4, 1) SK_ROWS(4, 2) SK_ROWS(4, 4) SK_ROWS(4, 8)
  SK_ROWS(8, 1) SK_ROWS(8, 2) SK_ROWS(8, 4) SK_ROWS(8, 8)
#undef SK_ROWS
  set_error("tsmttsm: no compiled row tile");
  return SKINNY_UNSUPPORTED;
}

template <typename T, typename Acc>
skinny_status tsmttsm_run(const DeviceInfo& dev, Workspace& ws, int* err, cudaStream_t st,
                          int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, T alpha,
                          const T* B, int64_t ldb, T beta, bool beta_zero, T* C, int64_t ldc,
                          const LaunchOpts& o) {
  const bool gram = (A == B) && (lda == ldb) && (M == N);
  if (rows_eligible<T, Acc>(M, N, gram, o))
    return tsmttsm_rows_run<T, Acc>(dev, ws, st, M, N, K, A, lda, alpha, B, ldb, beta, beta_zero, C, ldc, gram, o);
  TsmttsmPlan pl;
  skinny_status s = tsmttsm_plan<T, Acc>(dev, M, N, K, A, lda, B, ldb, gram, o, pl);
  if (s != SKINNY_OK) return s;
  s = workspace_ensure(ws, pl.partial_bytes, st);
  if (s != SKINNY_OK) return s;
  TsmttsmArgs<T> a;
  a.A = A;
  a.B = B;
  a.C = C;
  a.K = K;
  a.lda = lda;
  a.ldb = ldb;
  a.ldc = ldc;
  a.lda_s = pl.lda_s;
  a.ldb_s = pl.ldb_s;
  a.M = (int)M;
  a.N = (int)N;
  a.alpha = alpha;
  a.beta = beta;
  a.beta_zero = beta_zero;
  a.gram = gram;
  a.bulk = pl.bulk;
  a.rows = pl.rows;
  a.stages = pl.stages;
  a.ntiles = pl.ntiles;
  const int64_t sz = sizeof(T);
  a.bytes_a = (uint32_t)round_up(pl.rows * pl.lda_s * sz, 128);
  a.bytes_b = gram ? 0u : (uint32_t)round_up(pl.rows * pl.ldb_s * sz, 128);
  a.smem_avail = (uint32_t)(pl.smem - SMEM_HEADER);
  a.partials = ws.partials;
  a.counter = ws.counter;
  a.err = err;
  a.polls = dev.wait_polls;
  return tsmttsm_dispatch<T, Acc>(pl.tm, pl.tn, a, dim3(pl.grid, pl.groups), pl.smem, st);
}

// -------------------------------------------------------------------------------------- TSMM
template <typename T, typename Acc, int TN, int U>
skinny_status tsmm_launch_tile(const TsmmArgs<T>& a, int bps, int sms, int smem, cudaStream_t st) {
  static SmemAttr attr;
  auto kern = tsmm_kernel<T, Acc, TN, U>;
  ensure_smem_attr(kern, smem, attr);
  int occ = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, TSMM_THREADS, smem);
  if (occ < 1) occ = 1;
  if (bps > 0 && bps < occ) occ = bps;
  const int RS = TSMM_THREADS / a.gn * U;
  int64_t need = (a.K + RS - 1) / RS;
  int64_t grid = (int64_t)sms * occ;
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  kern<<<(int)grid, TSMM_THREADS, smem, st>>>(a);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("tsmm launch: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  return SKINNY_OK;
}

template <typename T, typename Acc>
skinny_status tsmm_run(const DeviceInfo& dev, cudaStream_t st, int64_t M, int64_t N, int64_t K,
                       const T* A, int64_t lda, T alpha, const T* B, int64_t ldb, T beta,
                       bool beta_zero, T* C, int64_t ldc, const LaunchOpts& o) {
  const int cap = sizeof(Acc) <= 8 ? 8 : (sizeof(Acc) <= 16 ? 4 : 2);
  int tn = pow2ceil(N) < cap ? pow2ceil(N) : cap;
  int gn = pow2ceil((N + tn - 1) / tn);
  if (gn > 32) {
    set_error("tsmm: N too large");
    return SKINNY_UNSUPPORTED;
  }
  const int np = gn * tn;
  const int64_t smem = (int64_t)M * np * sizeof(T);
  if (smem > dev.smem_optin) {
    set_error("tsmm: B does not fit in shared memory");
    return SKINNY_UNSUPPORTED;
  }
  TsmmArgs<T> a;
  a.A = A;
  a.B = B;
  a.C = C;
  a.K = K;
  a.lda = lda;
  a.ldb = ldb;
  a.ldc = ldc;
  a.M = (int)M;
  a.N = (int)N;
  a.alpha = alpha;
  a.beta = beta;
  a.beta_zero = beta_zero;
  // in place with M == N: C = A (alpha B + beta I), folded while B is staged
  a.fold = (const void*)A == (const void*)C && lda == ldc && M == N && !beta_zero && sizeof(Acc) == sizeof(T);
  a.gn = gn;
  a.np = np;
  const int sm = (int)(smem < 16 ? 16 : smem);
  // narrow rows (M <= 4, a few outputs per thread): 4 rows per thread and step
  // (32-byte accumulators: one row per thread and step)
  const bool multi = M <= 4 && tn <= 4 && sizeof(Acc) <= 16;
  switch (tn) {
    case 1:
      if constexpr (sizeof(Acc) <= 16)
        if (multi) return tsmm_launch_tile<T, Acc, 1, 4>(a, o.blocks_per_sm, dev.sms, sm, st);
      return tsmm_launch_tile<T, Acc, 1, 1>(a, o.blocks_per_sm, dev.sms, sm, st);
    case 2:
      if constexpr (sizeof(Acc) <= 16)
        if (multi) return tsmm_launch_tile<T, Acc, 2, 4>(a, o.blocks_per_sm, dev.sms, sm, st);
      return tsmm_launch_tile<T, Acc, 2, 1>(a, o.blocks_per_sm, dev.sms, sm, st);
    case 4:
      if constexpr (sizeof(Acc) <= 16) {
        return multi ? tsmm_launch_tile<T, Acc, 4, 4>(a, o.blocks_per_sm, dev.sms, sm, st)
                     : tsmm_launch_tile<T, Acc, 4, 1>(a, o.blocks_per_sm, dev.sms, sm, st);
      }
      break;
    default:
      if constexpr (sizeof(Acc) <= 8) return tsmm_launch_tile<T, Acc, 8, 1>(a, o.blocks_per_sm, dev.sms, sm, st);
  }
  set_error("tsmm: no compiled column tile");
  return SKINNY_UNSUPPORTED;
}

// Explicit instantiation of both launchers for a (storage, accumulator) pair (EXT empty: the
// inst_*.cu units, one pair or two each, so that the build compiles them in parallel) or its
// extern declaration (EXT extern: the units that call them).
#define SKINNY_LAUNCHERS(EXT, T, ACC)                                                                         \
  EXT template skinny_status tsmttsm_run<T, ACC>(const DeviceInfo&, Workspace&, int*, cudaStream_t, int64_t, \
                                                 int64_t, int64_t, const T*, int64_t, T, const T*, int64_t, T, \
                                                 bool, T*, int64_t, const LaunchOpts&);                      \
  EXT template skinny_status tsmm_run<T, ACC>(const DeviceInfo&, cudaStream_t, int64_t, int64_t, int64_t,     \
                                              const T*, int64_t, T, const T*, int64_t, T, bool, T*, int64_t,   \
                                              const LaunchOpts&);

}  // namespace skinny
