// split_complex.cu -- complex FP64 TSMTTSM in split precision (no counterpart in the reference,
// whose complex TSMTTSM is cuBLAS with OP_T, tsmttsm/gen_cublas.cuh:29-39).
//
// Interleaved complex A (K x M) and B (K x N) are real K x 2M and K x 2N matrices (columns
// re, im, re, im, ...).  Their real product P = A_r^T B_r (2M x 2N, split precision: split.cu
// for 2M, 2N <= 16, split_wide.cu up to 128) holds all four real products:
//   P[2n][2m] = ArT Br,  P[2n+1][2m+1] = AiT Bi,  P[2n+1][2m] = ArT Bi,  P[2n][2m+1] = AiT Br
// and C = alpha (P_rr - P_ii + i (P_ri + P_ir)) + beta C (plain transpose, as the reference), or
// alpha (P_rr + P_ii + i (P_ri - P_ir)) + beta C for the conjugate transpose A^H B.
// Each P entry carries the split kernels' accuracy; the combination adds FP64 roundings only.
#include <cstring>

#include "api_internal.h"

namespace skinny {

namespace {

constexpr int CMAX = 64;  // complex widths (real 128)

template <typename TO>
__global__ void combine_kernel(const double* __restrict__ P, int ldp, int M, int N, double ar, double ai, double br,
                               double bi, int beta_zero, int conj, TO* __restrict__ C, int64_t ldc) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= M * N) return;
  const int m = e % M, n = e / M;
  const double rr = P[(2 * n) * ldp + 2 * m], ii = P[(2 * n + 1) * ldp + 2 * m + 1];
  const double ri = P[(2 * n + 1) * ldp + 2 * m], ir = P[(2 * n) * ldp + 2 * m + 1];
  // A^T B: (rr - ii, ri + ir); A^H B (conjugated A): (rr + ii, ri - ir)
  const double sr = conj ? rr + ii : rr - ii, si = conj ? ri - ir : ri + ir;
  double vr = ar * sr - ai * si, vi = ar * si + ai * sr;
  TO* c = C + 2 * ((int64_t)n * ldc + m);
  if (!beta_zero) {
    const double cr = c[0], ci = c[1];
    vr += br * cr - bi * ci;
    vi += br * ci + bi * cr;
  }
  c[0] = (TO)vr;  // one rounding for complex FP32 storage
  c[1] = (TO)vi;
}

}  // namespace

skinny_status split_complex_tsmttsm(skinny_handle h, int64_t M, int64_t N, int64_t K, const void* A,
                                    int64_t lda, const void* alpha, const void* B, int64_t ldb,
                                    const void* beta, void* C, int64_t ldc, cudaStream_t st, bool autoselect,
                                    bool conj, bool f32) {
  if (M > CMAX || N > CMAX) {
    set_error("split precision complex TSMTTSM: M, N <= 64");
    return SKINNY_UNSUPPORTED;
  }
  void*& buf = h->split_ws[st];  // P, at most 128 x 128 doubles, one per stream
  if (!buf) {
    if (cudaMalloc(&buf, (size_t)4 * CMAX * CMAX * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      buf = nullptr;
      set_error("split complex: cudaMalloc failed");
      return SKINNY_NO_MEM;
    }
    h->extra_allocs.push_back(buf);
  }
  double* P = static_cast<double*>(buf);
  const double one = 1.0, zero = 0.0;
  // same buffer and leading dimension: the real product is a Gram product too
  skinny_status s = split_tsmttsm_t(h, f32, false, 2 * M, 2 * N, K, A, 2 * lda, &one, B, 2 * ldb, &zero, P, 2 * M,
                                    st, autoselect);
  if (s != SKINNY_OK) return s;
  double al[2], be[2];
  if (f32) {
    float af[2], bf[2];
    std::memcpy(af, alpha, sizeof af);
    std::memcpy(bf, beta, sizeof bf);
    al[0] = af[0], al[1] = af[1], be[0] = bf[0], be[1] = bf[1];
  } else {
    std::memcpy(al, alpha, sizeof al);
    std::memcpy(be, beta, sizeof be);
  }
  const int cells = (int)(M * N);
  const int bz = be[0] == 0.0 && be[1] == 0.0;
  if (f32)
    combine_kernel<float><<<(cells + 255) / 256, 256, 0, st>>>(P, (int)(2 * M), (int)M, (int)N, al[0], al[1], be[0],
                                                               be[1], bz, conj ? 1 : 0, static_cast<float*>(C), ldc);
  else
    combine_kernel<double><<<(cells + 255) / 256, 256, 0, st>>>(P, (int)(2 * M), (int)M, (int)N, al[0], al[1], be[0],
                                                                be[1], bz, conj ? 1 : 0, static_cast<double*>(C), ldc);
  count_launch();
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(std::string("split complex combine launch: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  return SKINNY_OK;
}

}  // namespace skinny
