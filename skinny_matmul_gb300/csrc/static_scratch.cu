// static_scratch.cu -- FP64 TSMTTSM entry point that allocates no device memory.
//
// skinny_tsmttsm_d_static() runs the same persistent TSMTTSM kernel as skinny_tsmttsm(R64,
// NATIVE), but its scratch (per-CTA partial sums, ticket counters, device error word) lives in
// the file-scope array below instead of a handle's cudaMalloc'ed workspace.  The array is part of
// the library's device image: every GPU that loads the library holds it until the process exits.
//
// Host code never passes the array's name to a kernel (in host code it is only a stand-in for
// the symbol); the first call on each device, with that device current, looks up the device
// address with cudaGetSymbolAddress and caches it.  Make that first call before any stream
// capture.  All calls share the one array: the ticket counters are cleared on the stream at every
// call, and calls that overlap on the GPU (different streams, or host threads racing) use the
// same partial buffer and race.  The error word is left alone by the calls: a bounded wait that
// timed out sets it, and skinny_tsmttsm_d_static_check() reads and clears it.
#include <cuda_runtime.h>

#include <mutex>

#include "api_internal.h"

namespace skinny {

extern template skinny_status tsmttsm_plan<double, double>(const DeviceInfo&, int64_t, int64_t,
                                                           int64_t, const void*, int64_t,
                                                           const void*, int64_t, bool,
                                                           const LaunchOpts&, TsmttsmPlan&);
extern template skinny_status tsmttsm_dispatch<double, double>(int, int, const TsmttsmArgs<double>&,
                                                               dim3, int, cudaStream_t);

constexpr size_t kStaticCounterBytes = 256;            // 64 ticket counters, cleared per call
constexpr size_t kStaticErrOffset = 256;               // device error word (bounded waits)
constexpr size_t kStaticHeaderBytes = 512;
constexpr size_t kStaticPartialBytes = (size_t)16 << 20;  // CTA partials: grid * M * N doubles
// Largest M * N: the CUDA-core kernel reduces through at most 64 groups of 256 cells of 8 x 8
// entries in FP64 (tsmttsm_plan), i.e. 2^20 entries of C; 2^20 * 8 bytes fills half the array,
// so at least two CTAs share the rows at the limit.
constexpr int64_t kStaticMaxCells = (int64_t)1 << 20;

static __device__ __align__(256) unsigned char g_tsmttsm_scratch[kStaticHeaderBytes + kStaticPartialBytes];

namespace {
struct StaticDevice {
  bool ready = false;
  unsigned char* base = nullptr;  // device address of g_tsmttsm_scratch on this device
  DeviceInfo info;
};
std::mutex g_static_mu;
StaticDevice g_static_dev[64];

skinny_status static_setup(int dev, StaticDevice*& out) {
  if (dev < 0 || dev >= 64) {
    set_error("static TSMTTSM: device index out of range");
    return SKINNY_BAD_ARG;
  }
  std::lock_guard<std::mutex> lk(g_static_mu);
  StaticDevice& s = g_static_dev[dev];
  if (!s.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_tsmttsm_scratch);  // device `dev` is current
    if (e != cudaSuccess || p == nullptr) {
      set_error(std::string("static TSMTTSM: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      cudaGetLastError();
      return SKINNY_DEVICE_ERROR;
    }
    s.base = static_cast<unsigned char*>(p);
    s.info.id = dev;
    cudaDeviceGetAttribute(&s.info.sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&s.info.smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    s.ready = true;
  }
  out = &s;
  return SKINNY_OK;
}
}  // namespace

}  // namespace skinny

using namespace skinny;

extern "C" skinny_status skinny_tsmttsm_d_static(int64_t M, int64_t N, int64_t K, const double* A,
                                                 int64_t lda, double alpha, const double* B,
                                                 int64_t ldb, double beta, double* C, int64_t ldc,
                                                 void* stream) {
  set_error("");
  skinny_status s = check_args(false, SKINNY_R64, M, N, K, A, lda, &alpha, B, ldb, &beta, C, ldc);
  if (s != SKINNY_OK) return s;
  if (M == 0 || N == 0) return SKINNY_OK;
  if (M * N > kStaticMaxCells) {
    set_error("static TSMTTSM: M*N exceeds the static scratch (at most 1048576 entries of C)");
    return SKINNY_BAD_ARG;
  }
  const size_t per_cta = (size_t)M * (size_t)N * sizeof(double);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    set_error("static TSMTTSM: no current CUDA device");
    return SKINNY_DEVICE_ERROR;
  }
  StaticDevice* sd = nullptr;
  s = static_setup(dev, sd);
  if (s != SKINNY_OK) return s;

  const bool gram = (A == B) && (lda == ldb) && (M == N);
  TsmttsmPlan pl;
  s = tsmttsm_plan<double, double>(sd->info, M, N, K, A, lda, B, ldb, gram, LaunchOpts{}, pl);
  if (s != SKINNY_OK) return s;
  const int64_t max_grid = (int64_t)(kStaticPartialBytes / per_cta);
  if (pl.grid > max_grid) pl.grid = (int)max_grid;  // fewer CTAs so the partials fit

  cudaStream_t st = (cudaStream_t)stream;
  // the ticket counters must start at zero; an earlier call that timed out leaves them behind
  if (cudaMemsetAsync(sd->base, 0, kStaticCounterBytes, st) != cudaSuccess) {
    cudaGetLastError();
    set_error("static TSMTTSM: clearing the scratch header failed");
    return SKINNY_DEVICE_ERROR;
  }
  TsmttsmArgs<double> a;
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
  a.beta_zero = beta == 0.0;
  a.gram = gram;
  a.bulk = pl.bulk;
  a.rows = pl.rows;
  a.stages = pl.stages;
  a.ntiles = pl.ntiles;
  a.bytes_a = (uint32_t)round_up(pl.rows * pl.lda_s * (int64_t)sizeof(double), 128);
  a.bytes_b = gram ? 0u : (uint32_t)round_up(pl.rows * pl.ldb_s * (int64_t)sizeof(double), 128);
  a.smem_avail = (uint32_t)(pl.smem - SMEM_HEADER);
  a.partials = sd->base + kStaticHeaderBytes;
  a.counter = reinterpret_cast<unsigned*>(sd->base);
  a.err = reinterpret_cast<int*>(sd->base + kStaticErrOffset);
  a.polls = kWaitPolls;
  return tsmttsm_dispatch<double, double>(pl.tm, pl.tn, a, dim3(pl.grid, pl.groups), pl.smem, st);
}

extern "C" skinny_status skinny_tsmttsm_d_static_check(void* stream) {
  set_error("");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    set_error("static TSMTTSM check: no current CUDA device");
    return SKINNY_DEVICE_ERROR;
  }
  StaticDevice* sd = nullptr;
  skinny_status s = static_setup(dev, sd);
  if (s != SKINNY_OK) return s;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  int flag = 0;
  if (e == cudaSuccess)
    e = cudaMemcpyFromSymbol(&flag, g_tsmttsm_scratch, sizeof(int), kStaticErrOffset, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    set_error(std::string("static TSMTTSM check: ") + cudaGetErrorString(e));
    cudaGetLastError();
    return SKINNY_DEVICE_ERROR;
  }
  if (flag == 0) return SKINNY_OK;
  const int zero = 0;
  if (cudaMemcpyToSymbol(g_tsmttsm_scratch, &zero, sizeof(int), kStaticErrOffset, cudaMemcpyHostToDevice) !=
      cudaSuccess) {
    cudaGetLastError();
    set_error("static TSMTTSM check: clearing the error word failed");
    return SKINNY_DEVICE_ERROR;
  }
  set_error("a bounded device-side wait of skinny_tsmttsm_d_static timed out");
  return SKINNY_TIMEOUT;
}
