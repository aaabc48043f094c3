// autotune.cu -- runtime selection of launch shapes and of the FP64 method per (op, dtype, M, N).
//
// The reference compiles one binary per (M, N, type) and picks kernels by fixed rules
// (versions.hpp:48-177, tsmm/fix_blend.cuh:7-29, tsmm/varip_blend.cuh:8-29).  Here the handle holds
// a table filled by measurement: for a key (op, dtype, acc, M, N) every candidate launch shape is
// timed on scratch operands with CUDA events and the fastest is kept.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"

namespace skinny {

__global__ void tune_fill_kernel(double* x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)(i * 2654435761u) ^ (uint32_t)(i >> 17);
    x[i] = (double)(h >> 8) * (1.0 / 16777216.0) - 0.5;
  }
}
__global__ void tune_fill_kernel_f(float* x, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)(i * 2654435761u) ^ (uint32_t)(i >> 17);
    x[i] = (float)(h >> 8) * (1.0f / 16777216.0f) - 0.5f;
  }
}

static void fill(void* p, size_t bytes, bool single, cudaStream_t st) {
  if (single)
    tune_fill_kernel_f<<<256, 256, 0, st>>>((float*)p, bytes / 4);
  else
    tune_fill_kernel<<<256, 256, 0, st>>>((double*)p, bytes / 8);
  count_launch();
}

static float time_one(skinny_handle h, bool tsmm, skinny_dtype dt, skinny_acc acc, int64_t M, int64_t N,
                      int64_t K, void* A, void* B, void* C, const LaunchOpts& o, cudaStream_t st,
                      skinny_status& status) {
  double one[2] = {1.0, 0.0}, half[2] = {0.5, 0.0};
  float onef[2] = {1.f, 0.f}, halff[2] = {0.5f, 0.f};
  const bool single = dt == SKINNY_R32 || dt == SKINNY_C32;
  const void* al = single ? (const void*)onef : (const void*)one;
  const void* be = single ? (const void*)halff : (const void*)half;
  const int64_t lda = M, ldb = tsmm ? M : N, ldc = tsmm ? N : M;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = -1.f;
  status = dispatch_product(h, tsmm, dt, acc, M, N, K, A, lda, al, B, ldb, be, C, ldc, st, o);
  for (int r = 0; r < 3 && status == SKINNY_OK; r++) {
    cudaEventRecord(e0, st);
    status = dispatch_product(h, tsmm, dt, acc, M, N, K, A, lda, al, B, ldb, be, C, ldc, st, o);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (best < 0.f || ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best * 1000.f;  // us
}

}  // namespace skinny

using namespace skinny;

extern "C" skinny_status skinny_autotune(skinny_handle h, int op, skinny_dtype dt, skinny_acc acc, int64_t M,
                                         int64_t N, int64_t K, void* stream) {
  set_error("");
  if (!h || (op != 0 && op != 1) || M < 1 || N < 1 || K < 1 || dtype_size(dt) == 0) {
    set_error("autotune: bad arguments");
    return SKINNY_BAD_ARG;
  }
  const bool tsmm = op == 1;
  DevGuard g(h->dev.id);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t s = dtype_size(dt);
  const bool single = dt == SKINNY_R32 || dt == SKINNY_C32;
  const size_t bA = (size_t)K * M * s, bB = (size_t)(tsmm ? M * N : K * N) * s,
               bC = (size_t)(tsmm ? K * N : M * N) * s;
  void *A = nullptr, *B = nullptr, *C = nullptr;
  if (cudaMalloc(&A, bA) != cudaSuccess || cudaMalloc(&B, bB) != cudaSuccess || cudaMalloc(&C, bC) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(A);
    cudaFree(B);
    cudaFree(C);
    set_error("autotune: scratch allocation failed");
    return SKINNY_NO_MEM;
  }
  fill(A, bA, single, st);
  fill(B, bB, single, st);
  fill(C, bC, single, st);

  std::vector<LaunchOpts> cands;
  if (tsmm) {
    for (int b : {0, 1, 2, 4}) cands.push_back(LaunchOpts{b, 0, -1});
  } else {
    for (int b : {1, 2})
      for (int r : {0, 64, 128, 256, 512}) cands.push_back(LaunchOpts{b, r, -1});
  }
  std::lock_guard<std::mutex> lk(h->mu);
  LaunchOpts best{};
  float best_us = -1.f;
  skinny_status status = SKINNY_OK;
  // the CUDA-core kernels (for AUTO on R64: the native method)
  const skinny_acc core = (acc == SKINNY_ACC_AUTO && dt == SKINNY_R64) ? SKINNY_ACC_NATIVE : acc;
  if (core != SKINNY_ACC_SPLIT) {
    for (const LaunchOpts& o : cands) {
      skinny_status st2;
      float us = time_one(h, tsmm, dt, core, M, N, K, A, B, C, o, st, st2);
      if (st2 == SKINNY_OK && us > 0.f && (best_us < 0.f || us < best_us)) {
        best_us = us;
        best = o;
        best.method = core;
      } else if (st2 != SKINNY_OK && st2 != SKINNY_UNSUPPORTED) {
        status = st2;
      }
    }
  }
  if (dt == SKINNY_R64 && (acc == SKINNY_ACC_AUTO || acc == SKINNY_ACC_SPLIT)) {
    skinny_status st2;
    LaunchOpts o{};
    float us = time_one(h, tsmm, dt, SKINNY_ACC_SPLIT, M, N, K, A, B, C, o, st, st2);
    if (st2 == SKINNY_OK && us > 0.f && (best_us < 0.f || us < best_us)) {
      best_us = us;
      best = o;
      best.method = SKINNY_ACC_SPLIT;
    }
  }
  cudaStreamSynchronize(st);
  cudaFree(A);
  cudaFree(B);
  cudaFree(C);
  if (best_us < 0.f) {
    set_error("autotune: no candidate ran");
    return status != SKINNY_OK ? status : SKINNY_UNSUPPORTED;
  }
  auto key = std::make_tuple((int)tsmm, (int)dt, (int)acc, M, N);
  h->tune[key] = best;
  h->tune_us[key] = best_us;
  return SKINNY_OK;
}

extern "C" skinny_status skinny_tune_export(skinny_handle h, char* buf, size_t len, size_t* written) {
  if (!h) return SKINNY_BAD_ARG;
  std::string out;
  {
    std::lock_guard<std::mutex> lk(h->mu);
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, h->dev.id);
    out = std::string("{\"device\": \"") + prop.name + "\", \"entries\": [\n";
    bool first = true;
    for (auto& kv : h->tune) {
      char line[256];
      const auto& k = kv.first;
      const LaunchOpts& o = kv.second;
      auto it = h->tune_us.find(k);
      std::snprintf(line, sizeof line,
                    "%s {\"op\": %d, \"dtype\": %d, \"acc\": %d, \"M\": %lld, \"N\": %lld, \"blocks_per_sm\": %d, "
                    "\"rows_per_tile\": %d, \"method\": %d, \"us\": %.3f}",
                    first ? "" : ",\n", std::get<0>(k), std::get<1>(k), std::get<2>(k), (long long)std::get<3>(k),
                    (long long)std::get<4>(k), o.blocks_per_sm, o.rows_per_tile, o.method,
                    it == h->tune_us.end() ? 0.0 : (double)it->second);
      out += line;
      first = false;
    }
    out += "\n]}\n";
  }
  if (written) *written = out.size() + 1;
  if (buf && len > 0) {
    std::strncpy(buf, out.c_str(), len);
    buf[len - 1] = 0;
    if (len < out.size() + 1) {
      set_error("tune_export: buffer too small");
      return SKINNY_BAD_ARG;
    }
  }
  return SKINNY_OK;
}

extern "C" skinny_status skinny_tune_import(skinny_handle h, const char* json) {
  if (!h || !json) return SKINNY_BAD_ARG;
  std::lock_guard<std::mutex> lk(h->mu);
  const char* p = json;
  int n = 0;
  while ((p = std::strstr(p, "{\"op\":")) != nullptr) {
    int op, dt, acc, bps, rows, method;
    long long M, N;
    double us;
    int got = std::sscanf(p,
                          "{\"op\": %d, \"dtype\": %d, \"acc\": %d, \"M\": %lld, \"N\": %lld, \"blocks_per_sm\": %d, "
                          "\"rows_per_tile\": %d, \"method\": %d, \"us\": %lf}",
                          &op, &dt, &acc, &M, &N, &bps, &rows, &method, &us);
    if (got != 9) {
      set_error("tune_import: malformed entry");
      return SKINNY_BAD_ARG;
    }
    auto key = std::make_tuple(op, dt, acc, (int64_t)M, (int64_t)N);
    h->tune[key] = LaunchOpts{bps, rows, method};
    h->tune_us[key] = (float)us;
    n++;
    p++;
  }
  return SKINNY_OK;
}
