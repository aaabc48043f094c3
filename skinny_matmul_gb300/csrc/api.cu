// api.cu -- the C ABI (include/skinny.h): handles, workspaces, argument checks, dispatch.
#include <cuda_runtime.h>

#include <atomic>
#include <climits>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "api_internal.h"
#include "launch.cuh"

namespace skinny {
// instantiated in the inst_*.cu units
SKINNY_LAUNCHERS(extern, float, float)
SKINNY_LAUNCHERS(extern, double, double)
SKINNY_LAUNCHERS(extern, double, dd)
SKINNY_LAUNCHERS(extern, c32, c32)
SKINNY_LAUNCHERS(extern, c64, c64)
SKINNY_LAUNCHERS(extern, c32h, c32h)
SKINNY_LAUNCHERS(extern, c64h, c64h)
SKINNY_LAUNCHERS(extern, float, double)
SKINNY_LAUNCHERS(extern, c32, c64)
SKINNY_LAUNCHERS(extern, c64, zdd)
}  // namespace skinny

namespace skinny {

static thread_local std::string g_last_error;
void set_error(const std::string& msg) { g_last_error = msg; }
static std::atomic<uint64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

skinny_status workspace_ensure(Workspace& ws, size_t bytes, cudaStream_t st) {
  if (!ws.counter) {
    if (cudaMalloc(&ws.counter, 256) != cudaSuccess) {
      cudaGetLastError();
      set_error("workspace: cudaMalloc of the ticket counter failed");
      return SKINNY_NO_MEM;
    }
    if (cudaMemsetAsync(ws.counter, 0, 256, st) != cudaSuccess) {
      set_error("workspace: cudaMemsetAsync failed");
      return SKINNY_DEVICE_ERROR;
    }
  }
  if (bytes <= ws.bytes) return SKINNY_OK;
  if (ws.partials) {
    cudaStreamSynchronize(st);  // earlier launches on this stream may still read the old buffer
    cudaFree(ws.partials);
    ws.partials = nullptr;
    ws.bytes = 0;
  }
  size_t nb = bytes < ((size_t)1 << 20) ? ((size_t)1 << 20) : bytes;
  if (cudaMalloc(&ws.partials, nb) != cudaSuccess) {
    cudaGetLastError();
    ws.partials = nullptr;
    set_error("workspace: cudaMalloc of " + std::to_string(nb) + " bytes failed");
    return SKINNY_NO_MEM;
  }
  ws.bytes = nb;
  return SKINNY_OK;
}

DevGuard::DevGuard(int d) {
  cudaGetDevice(&prev);
  changed = prev != d;
  if (changed) cudaSetDevice(d);
}
DevGuard::~DevGuard() {
  if (changed) cudaSetDevice(prev);
}

template <typename T>
static T load_scalar(const void* p) {
  T v;
  std::memcpy(&v, p, sizeof(T));
  return v;
}
static bool is_zero(float v) { return v == 0.f; }
static bool is_zero(double v) { return v == 0.0; }
static bool is_zero(c32 v) { return v.x == 0.f && v.y == 0.f; }
static bool is_zero(c64 v) { return v.x == 0.0 && v.y == 0.0; }
static bool is_zero(c32h v) { return v.x == 0.f && v.y == 0.f; }
static bool is_zero(c64h v) { return v.x == 0.0 && v.y == 0.0; }

size_t dtype_size(skinny_dtype dt) {
  switch (dt) {
    case SKINNY_R32: return 4;
    case SKINNY_R64: return 8;
    case SKINNY_C32: return 8;
    case SKINNY_C64: return 16;
  }
  return 0;
}

}  // namespace skinny

using namespace skinny;

skinny_handle_st::skinny_handle_st(int device) { dev.id = device; }

// ---------------------------------------------------------------------------------- handles
extern "C" skinny_status skinny_create(skinny_handle* handle, int device) {
  if (!handle) {
    set_error("skinny_create: null handle pointer");
    return SKINNY_BAD_ARG;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    set_error("skinny_create: no such CUDA device");
    return SKINNY_BAD_ARG;
  }
  DevGuard g(device);
  skinny_handle h = new skinny_handle_st(device);
  cudaDeviceGetAttribute(&h->dev.sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&h->dev.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  if (cudaMalloc(&h->err, 64) != cudaSuccess || cudaMemset(h->err, 0, 64) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    set_error("skinny_create: cudaMalloc failed");
    return SKINNY_NO_MEM;
  }
  *handle = h;
  return SKINNY_OK;
}

extern "C" skinny_status skinny_destroy(skinny_handle h) {
  if (!h) return SKINNY_BAD_ARG;
  {
    DevGuard g(h->dev.id);
    cudaDeviceSynchronize();
    for (auto& kv : h->ws) {
      if (kv.second.partials) cudaFree(kv.second.partials);
      if (kv.second.counter) cudaFree(kv.second.counter);
    }
    for (void* p : h->extra_allocs) cudaFree(p);
    if (h->err) cudaFree(h->err);
    group_release(h);
  }
  delete h;
  return SKINNY_OK;
}

extern "C" const char* skinny_status_string(skinny_status s) {
  switch (s) {
    case SKINNY_OK: return "SKINNY_OK";
    case SKINNY_UNSUPPORTED: return "SKINNY_UNSUPPORTED";
    case SKINNY_BAD_ARG: return "SKINNY_BAD_ARG";
    case SKINNY_NO_MEM: return "SKINNY_NO_MEM";
    case SKINNY_TIMEOUT: return "SKINNY_TIMEOUT";
    case SKINNY_DEVICE_ERROR: return "SKINNY_DEVICE_ERROR";
    case SKINNY_NOT_READY: return "SKINNY_NOT_READY";
  }
  return "SKINNY_UNKNOWN";
}

extern "C" const char* skinny_last_error(void) { return g_last_error.c_str(); }

extern "C" uint64_t skinny_kernel_launches(void) { return g_launches.load(); }

extern "C" skinny_status skinny_check_device(skinny_handle h) {
  if (!h) return SKINNY_BAD_ARG;
  DevGuard g(h->dev.id);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    set_error(std::string("device: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  int flag = 0;
  cudaMemcpy(&flag, h->err, sizeof(int), cudaMemcpyDeviceToHost);
  if (flag == 0) return SKINNY_OK;
  cudaMemset(h->err, 0, 64);
  std::lock_guard<std::mutex> lk(h->mu);
  for (auto& kv : h->ws)
    if (kv.second.counter) cudaMemset(kv.second.counter, 0, 256);
  cudaDeviceSynchronize();
  set_error("a bounded device-side wait timed out");
  return SKINNY_TIMEOUT;
}

extern "C" skinny_status skinny_set_wait_limit(skinny_handle h, uint32_t polls) {
  if (!h) return SKINNY_BAD_ARG;
  std::lock_guard<std::mutex> lk(h->mu);
  h->dev.wait_polls = polls;
  return SKINNY_OK;
}

// ---------------------------------------------------------------------------------- products
namespace skinny {

template <typename T, typename Acc>
static skinny_status run_t(skinny_handle h, bool tsmm, int64_t M, int64_t N, int64_t K,
                           const void* A, int64_t lda, const void* alpha, const void* B, int64_t ldb,
                           const void* beta, void* C, int64_t ldc, cudaStream_t st,
                           const LaunchOpts& o) {
  T al = load_scalar<T>(alpha), be = load_scalar<T>(beta);
  const bool bz = is_zero(be);
  if (tsmm)
    return tsmm_run<T, Acc>(h->dev, st, M, N, K, (const T*)A, lda, al, (const T*)B, ldb, be, bz,
                            (T*)C, ldc, o);
  Workspace& ws = h->ws[st];
  return tsmttsm_run<T, Acc>(h->dev, ws, h->err, st, M, N, K, (const T*)A, lda, al, (const T*)B,
                             ldb, be, bz, (T*)C, ldc, o);
}

skinny_status check_args(bool tsmm, skinny_dtype dt, int64_t M, int64_t N, int64_t K,
                         const void* A, int64_t lda, const void* alpha, const void* B,
                         int64_t ldb, const void* beta, const void* C, int64_t ldc) {
  if (dtype_size(dt) == 0) {
    set_error("unknown dtype");
    return SKINNY_BAD_ARG;
  }
  if (M < 0 || N < 0 || K < 0 || M > INT_MAX || N > INT_MAX) {
    set_error("negative or oversized M, N, K");
    return SKINNY_BAD_ARG;
  }
  if (!alpha || !beta) {
    set_error("alpha / beta must point to host scalars");
    return SKINNY_BAD_ARG;
  }
  if (lda < (M > 1 ? M : 1) || ldb < ((tsmm ? M : N) > 1 ? (tsmm ? M : N) : 1) ||
      ldc < ((tsmm ? N : M) > 1 ? (tsmm ? N : M) : 1)) {
    set_error("leading dimension smaller than the row width");
    return SKINNY_BAD_ARG;
  }
  if ((K > 0 && M > 0 && N > 0 && (!A || !B)) || (M > 0 && N > 0 && !C)) {
    set_error("null device pointer");
    return SKINNY_BAD_ARG;
  }
  if (tsmm && A == C && lda != ldc) {
    set_error("in-place TSMM (A == C) requires lda == ldc");
    return SKINNY_BAD_ARG;
  }
  if (!tsmm && (C == A || C == B) && K > 0) {
    set_error("TSMTTSM output must not alias an input");
    return SKINNY_BAD_ARG;
  }
  return SKINNY_OK;
}

skinny_status dispatch_product(skinny_handle h, bool tsmm, skinny_dtype dt, skinny_acc acc,
                               int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                               const void* alpha, const void* B, int64_t ldb, const void* beta,
                               void* C, int64_t ldc, cudaStream_t st, const LaunchOpts& o) {
  switch (dt) {
    case SKINNY_R32:
      if (acc == SKINNY_ACC_DD)  // FP64 accumulation of exact products
        return run_t<float, double>(h, tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
      if (acc == SKINNY_ACC_SPLIT)  // exact products on the tensor cores
        return tsmm ? split_tsmm_t(h, false, true, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, false)
                    : split_tsmttsm_t(h, true, true, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, false);
      if (acc == SKINNY_ACC_NATIVE || acc == SKINNY_ACC_AUTO)
        return run_t<float, float>(h, tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
      break;
    case SKINNY_R64:
      if (acc == SKINNY_ACC_DD)
        return run_t<double, dd>(h, tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
      if (acc == SKINNY_ACC_AUTO && o.method == SKINNY_ACC_NATIVE)
        return run_t<double, double>(h, tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
      if (acc == SKINNY_ACC_SPLIT || acc == SKINNY_ACC_AUTO) {
        // a tuned SPLIT entry forces the split kernel; otherwise AUTO uses its measured heuristic
        skinny_status s = split_product(h, tsmm, M, N, K, (const double*)A, lda, alpha,
                                        (const double*)B, ldb, beta, (double*)C, ldc, st,
                                        acc == SKINNY_ACC_AUTO && o.method != SKINNY_ACC_SPLIT);
        if (s != SKINNY_UNSUPPORTED || acc == SKINNY_ACC_SPLIT) return s;
      }
      return run_t<double, double>(h, tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
    case SKINNY_C32:
      if (acc == SKINNY_ACC_DD)  // complex FP64 accumulation of exact products
        return run_t<c32, c64>(h, tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
      if (acc == SKINNY_ACC_SPLIT)
        return tsmm ? split_tsmm_t(h, true, true, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, false)
                    : split_complex_tsmttsm(h, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, false, false, true);
      if (acc == SKINNY_ACC_NATIVE || acc == SKINNY_ACC_AUTO)
        return run_t<c32, c32>(h, tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
      break;
    case SKINNY_C64:
      if (acc == SKINNY_ACC_DD)  // double-double real and imaginary parts
        return run_t<c64, zdd>(h, tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
      if (acc == SKINNY_ACC_SPLIT || (acc == SKINNY_ACC_AUTO && o.method != SKINNY_ACC_NATIVE)) {
        const bool autosel = acc == SKINNY_ACC_AUTO && o.method != SKINNY_ACC_SPLIT;
        skinny_status s =
            tsmm ? split_tsmm(h, true, M, N, K, (const double*)A, lda, alpha, (const double*)B, ldb, beta,
                              (double*)C, ldc, st, autosel)
                 : split_complex_tsmttsm(h, M, N, K, A, lda, alpha, B, ldb, beta,
                                         (double*)C, ldc, st, autosel);
        if (s != SKINNY_UNSUPPORTED || acc == SKINNY_ACC_SPLIT) return s;
      }
      if (acc == SKINNY_ACC_NATIVE || acc == SKINNY_ACC_AUTO)
        return run_t<c64, c64>(h, tsmm, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
      break;
  }
  set_error("method not provided for this dtype");
  return SKINNY_UNSUPPORTED;
}

skinny_status product(skinny_handle h, bool tsmm, skinny_dtype dt, skinny_acc acc, int64_t M,
                      int64_t N, int64_t K, const void* A, int64_t lda, const void* alpha,
                      const void* B, int64_t ldb, const void* beta, void* C, int64_t ldc,
                      void* stream, const LaunchOpts* opts) {
  set_error("");
  if (!h) {
    set_error("null handle");
    return SKINNY_BAD_ARG;
  }
  skinny_status s = check_args(tsmm, dt, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc);
  if (s != SKINNY_OK) return s;
  if (M == 0 || N == 0 || (tsmm && K == 0)) return SKINNY_OK;
  DevGuard g(h->dev.id);
  cudaStream_t st = (cudaStream_t)stream;
  LaunchOpts o = opts ? *opts : h->tuned(tsmm, dt, acc, M, N);
  std::lock_guard<std::mutex> lk(h->mu);
  return dispatch_product(h, tsmm, dt, acc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
}

}  // namespace skinny

extern "C" skinny_status skinny_tsmttsm(skinny_handle h, skinny_dtype dt, skinny_acc acc,
                                        int64_t M, int64_t N, int64_t K, const void* A,
                                        int64_t lda, const void* alpha, const void* B,
                                        int64_t ldb, const void* beta, void* C, int64_t ldc,
                                        void* stream) {
  return product(h, false, dt, acc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, stream, nullptr);
}

extern "C" skinny_status skinny_tsmm(skinny_handle h, skinny_dtype dt, skinny_acc acc, int64_t M,
                                     int64_t N, int64_t K, const void* A, int64_t lda,
                                     const void* alpha, const void* B, int64_t ldb,
                                     const void* beta, void* C, int64_t ldc, void* stream) {
  return product(h, true, dt, acc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, stream, nullptr);
}

namespace skinny {
skinny_status dispatch_conj(skinny_handle h, skinny_dtype dt, skinny_acc acc, int64_t M, int64_t N, int64_t K,
                            const void* A, int64_t lda, const void* alpha, const void* B, int64_t ldb,
                            const void* beta, void* C, int64_t ldc, cudaStream_t st) {
  LaunchOpts o{};
  if (dt == SKINNY_C64 && (acc == SKINNY_ACC_SPLIT || acc == SKINNY_ACC_AUTO)) {
    skinny_status s = split_complex_tsmttsm(h, M, N, K, A, lda, alpha, B, ldb, beta,
                                            (double*)C, ldc, st, acc == SKINNY_ACC_AUTO, true);
    if (s != SKINNY_UNSUPPORTED || acc == SKINNY_ACC_SPLIT) return s;
  }
  if (acc != SKINNY_ACC_NATIVE && acc != SKINNY_ACC_AUTO) {
    set_error("method not provided for this dtype");
    return SKINNY_UNSUPPORTED;
  }
  if (dt == SKINNY_C32) return run_t<c32h, c32h>(h, false, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
  return run_t<c64h, c64h>(h, false, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, st, o);
}
}  // namespace skinny

// C = alpha A^H B + beta C (conjugate transpose; the reference has only the plain transpose,
// tsmttsm/gen_cublas.cuh:29-39).  Real dtypes: the same as skinny_tsmttsm.
extern "C" skinny_status skinny_tsmttsm_conj(skinny_handle h, skinny_dtype dt, skinny_acc acc, int64_t M,
                                             int64_t N, int64_t K, const void* A, int64_t lda,
                                             const void* alpha, const void* B, int64_t ldb,
                                             const void* beta, void* C, int64_t ldc, void* stream) {
  if (dt == SKINNY_R32 || dt == SKINNY_R64)
    return product(h, false, dt, acc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, stream, nullptr);
  set_error("");
  if (!h) {
    set_error("null handle");
    return SKINNY_BAD_ARG;
  }
  skinny_status s = check_args(false, dt, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc);
  if (s != SKINNY_OK) return s;
  if (M == 0 || N == 0) return SKINNY_OK;
  DevGuard g(h->dev.id);
  std::lock_guard<std::mutex> lk(h->mu);
  return dispatch_conj(h, dt, acc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc, (cudaStream_t)stream);
}

// ----------------------------------------------------------------- reference-shaped wrappers
skinny_handle skinny::default_handle() {
  static std::mutex mu;
  static std::map<int, skinny_handle> hs;
  int d = 0;
  cudaGetDevice(&d);
  std::lock_guard<std::mutex> lk(mu);
  auto it = hs.find(d);
  if (it != hs.end()) return it->second;
  skinny_handle h = nullptr;
  if (skinny_create(&h, d) != SKINNY_OK) return nullptr;
  hs[d] = h;
  return h;
}

#define SK_REF(NAME, OPTSMM, DT, ACC, T, HT)                                                         \
  extern "C" int NAME(size_t blockCount, int M, int N, int K, const T* A, int lda, HT alpha,       \
                      const T* B, int ldb, HT beta, T* C, int ldc) {                               \
    (void)blockCount;                                                                              \
    skinny_handle h = default_handle();                                                            \
    if (!h) return 0;                                                                              \
    return product(h, OPTSMM, DT, ACC, M, N, K, A, lda, &alpha, B, ldb, &beta, C, ldc, nullptr,    \
                   nullptr) == SKINNY_OK;                                                          \
  }

SK_REF(skinny_tsmttsm_s, false, SKINNY_R32, SKINNY_ACC_NATIVE, float, float)
SK_REF(skinny_tsmttsm_d, false, SKINNY_R64, SKINNY_ACC_NATIVE, double, double)
SK_REF(skinny_tsmttsm_c, false, SKINNY_C32, SKINNY_ACC_NATIVE, skinny_c32, skinny_c32)
SK_REF(skinny_tsmttsm_z, false, SKINNY_C64, SKINNY_ACC_NATIVE, skinny_c64, skinny_c64)
SK_REF(skinny_tsmttsm_dd, false, SKINNY_R64, SKINNY_ACC_DD, double, double)
SK_REF(skinny_tsmm_s, true, SKINNY_R32, SKINNY_ACC_NATIVE, float, float)
SK_REF(skinny_tsmm_d, true, SKINNY_R64, SKINNY_ACC_NATIVE, double, double)
SK_REF(skinny_tsmm_c, true, SKINNY_C32, SKINNY_ACC_NATIVE, skinny_c32, skinny_c32)
SK_REF(skinny_tsmm_z, true, SKINNY_C64, SKINNY_ACC_NATIVE, skinny_c64, skinny_c64)
SK_REF(skinny_tsmm_dd, true, SKINNY_R64, SKINNY_ACC_DD, double, double)
#undef SK_REF
