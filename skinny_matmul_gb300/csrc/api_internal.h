// api_internal.h -- handle layout and internal entry points shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "launch.cuh"
#include "skinny.h"

struct skinny_handle_st {
  explicit skinny_handle_st(int device);
  skinny::DeviceInfo dev;
  std::mutex mu;                                        // guards ws / tune / extra state
  std::map<cudaStream_t, skinny::Workspace> ws;         // one partial-sum buffer per stream
  std::map<std::tuple<int, int, int, int64_t, int64_t>, skinny::LaunchOpts> tune;  // autotuner table
  std::map<std::tuple<int, int, int, int64_t, int64_t>, float> tune_us;            // measured time
  std::vector<void*> extra_allocs;                       // buffers owned by other subsystems
  std::map<cudaStream_t, void*> split_ws;                // split-precision scratch per stream
  std::map<cudaStream_t, size_t> split_ws_bytes;
  std::map<cudaStream_t, void*> svqb_ws;                 // SVQB scratch per stream
  std::map<cudaStream_t, void*> svqbz_ws;                // complex SVQB scratch per stream
  int* err = nullptr;                                    // device error word (bounded waits)

  // launch options recorded by the autotuner for (op, dtype, acc, M, N); defaults otherwise
  skinny::LaunchOpts tuned(bool tsmm, skinny_dtype dt, skinny_acc acc, int64_t M, int64_t N) {
    std::lock_guard<std::mutex> lk(mu);
    auto it = tune.find(std::make_tuple((int)tsmm, (int)dt, (int)acc, M, N));
    return it == tune.end() ? skinny::LaunchOpts{} : it->second;
  }
};

namespace skinny {

struct DevGuard {
  explicit DevGuard(int d);
  ~DevGuard();
  int prev = 0;
  bool changed = false;
};

size_t dtype_size(skinny_dtype dt);
skinny_handle default_handle();

skinny_status check_args(bool tsmm, skinny_dtype dt, int64_t M, int64_t N, int64_t K,
                         const void* A, int64_t lda, const void* alpha, const void* B,
                         int64_t ldb, const void* beta, const void* C, int64_t ldc);

// Full product entry (argument checks, device guard, handle lock, dispatch).
skinny_status product(skinny_handle h, bool tsmm, skinny_dtype dt, skinny_acc acc, int64_t M,
                      int64_t N, int64_t K, const void* A, int64_t lda, const void* alpha,
                      const void* B, int64_t ldb, const void* beta, void* C, int64_t ldc,
                      void* stream, const LaunchOpts* opts);

// Dispatch without checks or locking (caller holds h->mu and the device guard).
skinny_status dispatch_product(skinny_handle h, bool tsmm, skinny_dtype dt, skinny_acc acc,
                               int64_t M, int64_t N, int64_t K, const void* A, int64_t lda,
                               const void* alpha, const void* B, int64_t ldb, const void* beta,
                               void* C, int64_t ldc, cudaStream_t st, const LaunchOpts& o);

// C = alpha A^H B + beta C for complex dtypes without checks or locking (caller holds h->mu).
skinny_status dispatch_conj(skinny_handle h, skinny_dtype dt, skinny_acc acc, int64_t M, int64_t N, int64_t K,
                            const void* A, int64_t lda, const void* alpha, const void* B, int64_t ldb,
                            const void* beta, void* C, int64_t ldc, cudaStream_t st);

// FP64 split-precision (tensor-core) products; SKINNY_UNSUPPORTED when the shape is not covered
// (for auto == true the caller then falls back to the CUDA-core FP64 kernels).
skinny_status split_product(skinny_handle h, bool tsmm, int64_t M, int64_t N, int64_t K,
                            const double* A, int64_t lda, const void* alpha, const double* B,
                            int64_t ldb, const void* beta, double* C, int64_t ldc,
                            cudaStream_t st, bool autoselect);

// TSMTTSM in split precision with FP32 storage as well (split.cu): in_f32 reads A and B as FP32
// (widened exactly), out_f32 writes C (and takes alpha, beta) as FP32; M, N <= 128.
skinny_status split_tsmttsm_t(skinny_handle h, bool in_f32, bool out_f32, int64_t M, int64_t N, int64_t K,
                              const void* A, int64_t lda, const void* alpha, const void* B, int64_t ldb,
                              const void* beta, void* C, int64_t ldc, cudaStream_t st, bool autoselect);

// FP64 TSMTTSM in split precision for M or N in 17..128 (split_wide.cu); SKINNY_UNSUPPORTED beyond.
skinny_status split_wide(skinny_handle h, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                         const void* alpha, const double* B, int64_t ldb, const void* beta, double* C,
                         int64_t ldc, cudaStream_t st);
// The same with FP32 inputs (in_f32) and / or FP32 output, alpha and beta (out_f32).
skinny_status split_wide_t(skinny_handle h, bool in_f32, bool out_f32, int64_t M, int64_t N, int64_t K,
                           const void* A, int64_t lda, const void* alpha, const void* B, int64_t ldb,
                           const void* beta, void* C, int64_t ldc, cudaStream_t st);

// Complex FP64 TSMTTSM in split precision through the real product of doubled width
// (split_complex.cu); M, N <= 64.  f32: complex FP32 storage (A, B, C, alpha, beta).
skinny_status split_complex_tsmttsm(skinny_handle h, int64_t M, int64_t N, int64_t K, const void* A,
                                    int64_t lda, const void* alpha, const void* B, int64_t ldb,
                                    const void* beta, void* C, int64_t ldc, cudaStream_t st, bool autoselect,
                                    bool conj = false, bool f32 = false);

// FP64 / complex FP64 TSMM in split precision (split_tsmm.cu); SKINNY_UNSUPPORTED outside its range.
skinny_status split_tsmm(skinny_handle h, bool cplx, int64_t M, int64_t N, int64_t K, const double* A,
                         int64_t lda, const void* alpha, const double* B, int64_t ldb, const void* beta, double* C,
                         int64_t ldc, cudaStream_t st, bool autoselect);
// The same for FP32 / complex FP32 storage as well (f32: A, B, C, alpha, beta are float): values
// widened exactly to FP64 in registers, the result rounded once to FP32 after beta * C in FP64.
skinny_status split_tsmm_t(skinny_handle h, bool cplx, bool f32, int64_t M, int64_t N, int64_t K, const void* A,
                           int64_t lda, const void* alpha, const void* B, int64_t ldb, const void* beta, void* C,
                           int64_t ldc, cudaStream_t st, bool autoselect);

// Frees the grouped-launch buffers owned by a handle (group.cu).
void group_release(skinny_handle h);

}  // namespace skinny
