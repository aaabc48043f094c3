// svqb.cu -- SVQB orthogonalisation entirely on the device.
//
// Follows svqb/svqb.cu:72-130 of the reference step by step, but keeps every step on the GPU
// (the reference copies S to the host and calls MAGMA's dsyevd there, svqb.cu:95-120):
//   1. S = X^T X                      TSMTTSM in Gram mode, method chosen by the caller
//   2. d_i = 1/sqrt(S_ii) if |S_ii| > 1e-15 else 0;  S <- D S D        (svqb.cu:99-110)
//   3. S = U L U^T                    one-CTA cyclic Jacobi in FP64 (parallel round-robin order:
//                                     the M/2 rotations of a round at once), eigenvalues
//                                     ascending as dsyevd returns them
//   4. T = D U diag(1/sqrt(max(1e-15, l)))  stored as TSMM's B (B[n*M+m])  (svqb.cu:115-119)
//   5. X <- X T                       in-place TSMM                      (svqb.cu:124-129)
//   6. optional ||Q^T Q - I||_F with a double-double Gram                (svqb.cu:184-211)
// Eigenvector signs are fixed so that the largest-magnitude entry of each is positive.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "api_internal.h"

namespace skinny {

constexpr int SVQB_MAX_M = 64;
constexpr int SVQB_THREADS = 256;

// Jacobi on the scaled Gram matrix; writes T (B layout of TSMM) and the sweep count.
__global__ void __launch_bounds__(SVQB_THREADS) svqb_eig_kernel(const double* __restrict__ S, int M,
                                                                double* __restrict__ T, int* info,
                                                                int max_sweeps) {
  extern __shared__ __align__(16) double sh[];
  const int LD = M + 1;
  double* A = sh;                 // M x LD
  double* V = A + M * LD;         // M x LD
  double* d = V + M * LD;         // M
  double* cs = d + M;             // 2 * (M/2 + 1)
  double* red = cs + 2 * (M / 2 + 1);  // SVQB_THREADS
  int* order = reinterpret_cast<int*>(red + SVQB_THREADS);  // M
  int* pq = order + SVQB_MAX_M;                             // 2 * (M/2 + 1): the round's pairs
  const int tid = threadIdx.x;
  // rotation work: thread = (pair lane k0, row / column i0); no division by runtime values
  constexpr int KS = SVQB_THREADS / SVQB_MAX_M;
  const int i0 = tid % SVQB_MAX_M, k0 = tid / SVQB_MAX_M;

  for (int i = tid; i < M; i += SVQB_THREADS) {
    double sii = S[i * M + i];
    d[i] = fabs(sii) > 1.0e-15 ? 1.0 / sqrt(sii) : 0.0;
  }
  __syncthreads();
  for (int e = tid; e < M * M; e += SVQB_THREADS) {
    int i = e / M, j = e % M;
    A[i * LD + j] = S[i * M + j] * d[i] * d[j];
    V[i * LD + j] = (i == j) ? 1.0 : 0.0;
  }
  __syncthreads();

  const int n = (M + 1) & ~1;  // players of the round-robin (a dummy when M is odd)
  const int npairs = n / 2;
  // converged when the off-diagonal mass is at the rounding level of the matrix ((M u)^2 of the
  // whole), or when it is small and a sweep no longer reduces it (rounding noise)
  const double tol = (double)M * M * 1.23e-32;
  double prev_off = 0.0;
  int sweeps = 0;
  for (; sweeps < max_sweeps; sweeps++) {
    // convergence: off-diagonal mass relative to the whole matrix
    double off = 0.0, all = 0.0;
    for (int e = tid; e < M * M; e += SVQB_THREADS) {
      int i = e / M, j = e % M;
      double a = A[i * LD + j];
      all += a * a;
      if (i != j) off += a * a;
    }
    red[tid] = off;
    __syncthreads();
    for (int s = SVQB_THREADS / 2; s > 0; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    const double off_sum = red[0];
    __syncthreads();
    red[tid] = all;
    __syncthreads();
    for (int s = SVQB_THREADS / 2; s > 0; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    const double all_sum = red[0];
    __syncthreads();
    if (off_sum <= tol * all_sum || M == 1 || (sweeps > 0 && off_sum <= 1.0e-20 * all_sum && off_sum >= 0.25 * prev_off))
      break;
    prev_off = off_sum;

    for (int r = 0; r < n - 1; r++) {
      // pair k: (n-1, r) for k = 0, ((r+k) % (n-1), (r-k+n-1) % (n-1)) otherwise; the rotation
      // of each pair and the pair itself go to shared memory once per round
      for (int k = tid; k < npairs; k += SVQB_THREADS) {
        int p = k == 0 ? n - 1 : (r + k) % (n - 1);
        int q = k == 0 ? r : (r - k + n - 1) % (n - 1);
        if (p > q) {
          int x = p;
          p = q;
          q = x;
        }
        double c = 1.0, s = 0.0;
        if (q < M) {
          const double apq = A[p * LD + q];
          if (apq != 0.0) {
            const double tau = (A[q * LD + q] - A[p * LD + p]) / (2.0 * apq);
            const double t = tau >= 0.0 ? 1.0 / (tau + sqrt(1.0 + tau * tau)) : -1.0 / (-tau + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        } else {
          q = p;  // the dummy player: an identity rotation on p
        }
        cs[2 * k] = c;
        cs[2 * k + 1] = s;
        pq[2 * k] = p;
        pq[2 * k + 1] = q;
      }
      __syncthreads();
      // A <- A J, V <- V J (column rotations): thread (k0, i) takes row i of pairs k0, k0 + KS, ...
      if (i0 < M)
        for (int k = k0; k < npairs; k += KS) {
          const int p = pq[2 * k], q = pq[2 * k + 1];
          if (p == q) continue;
          const double c = cs[2 * k], s = cs[2 * k + 1];
          const double aip = A[i0 * LD + p], aiq = A[i0 * LD + q];
          A[i0 * LD + p] = c * aip - s * aiq;
          A[i0 * LD + q] = s * aip + c * aiq;
          const double vip = V[i0 * LD + p], viq = V[i0 * LD + q];
          V[i0 * LD + p] = c * vip - s * viq;
          V[i0 * LD + q] = s * vip + c * viq;
        }
      __syncthreads();
      // A <- J^T A (row rotations): thread (k0, j) takes column j
      if (i0 < M)
        for (int k = k0; k < npairs; k += KS) {
          const int p = pq[2 * k], q = pq[2 * k + 1];
          if (p == q) continue;
          const double c = cs[2 * k], s = cs[2 * k + 1];
          const double apj = A[p * LD + i0], aqj = A[q * LD + i0];
          A[p * LD + i0] = c * apj - s * aqj;
          A[q * LD + i0] = s * apj + c * aqj;
        }
      __syncthreads();
    }
  }

  // ascending eigenvalues: rank of each diagonal entry (ties broken by index)
  for (int i = tid; i < M; i += SVQB_THREADS) {
    const double li = A[i * LD + i];
    int rank = 0;
    for (int j = 0; j < M; j++) {
      const double lj = A[j * LD + j];
      rank += (lj < li) || (lj == li && j < i);
    }
    order[rank] = i;
  }
  __syncthreads();
  // T[col*M + m] = V[m][src] * d[m] / sqrt(max(1e-15, l_src)), sign: largest |V[.][src]| positive
  for (int col = tid; col < M; col += SVQB_THREADS) {
    const int src = order[col];
    double big = 0.0, sg = 1.0;
    for (int m = 0; m < M; m++) {
      const double v = V[m * LD + src];
      if (fabs(v) > big) {
        big = fabs(v);
        sg = v < 0.0 ? -1.0 : 1.0;
      }
    }
    const double lam = A[src * LD + src];
    const double f = sg / sqrt(fmax(1.0e-15, lam));
    for (int m = 0; m < M; m++) T[col * M + m] = V[m * LD + src] * d[m] * f;
  }
  if (tid == 0 && info) *info = sweeps;
}

// ||S - I||_F for an M x M matrix
__global__ void __launch_bounds__(SVQB_THREADS) svqb_orth_kernel(const double* __restrict__ S, int M, double* out) {
  __shared__ double red[SVQB_THREADS];
  double acc = 0.0;
  for (int e = threadIdx.x; e < M * M; e += SVQB_THREADS) {
    const int i = e / M, j = e % M;
    const double v = (i == j ? 1.0 : 0.0) - S[e];
    acc += v * v;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = SVQB_THREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sqrt(red[0]);
}

// Cholesky S = R^T R (R upper, positive diagonal) of the Gram matrix and T = R^-1 in TSMM's B
// layout (B[n*M + m] = Rinv[m][n]), so that X <- X T gives Q = X R^-1.  *info = 0, or j + 1 when
// the pivot of column j is not positive (the Gram is not numerically positive definite).
__global__ void __launch_bounds__(SVQB_THREADS) cholqr_kernel(const double* __restrict__ S, int M,
                                                              double* __restrict__ T, int* info) {
  extern __shared__ __align__(16) double sh[];
  const int LD = M + 1;
  double* A = sh;         // M x LD: the trailing matrix, then R in the upper triangle
  double* Y = A + M * LD;  // M x LD: R^-1
  __shared__ int bad;
  const int tid = threadIdx.x;
  for (int e = tid; e < M * M; e += SVQB_THREADS) A[(e / M) * LD + e % M] = S[e];
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < M; j++) {
    const double piv = A[j * LD + j];
    if (!(piv > 0.0)) {  // uniform: every thread reads the same pivot
      if (tid == 0) bad = j + 1;
      break;
    }
    const double r = sqrt(piv);
    __syncthreads();
    for (int i = j + 1 + tid; i < M; i += SVQB_THREADS) A[j * LD + i] /= r;  // row j of R
    if (tid == 0) A[j * LD + j] = r;
    __syncthreads();
    // trailing update A[i][l] -= R[j][i] R[j][l] for j < i <= l
    const int w = M - j - 1;
    for (int e = tid; e < w * w; e += SVQB_THREADS) {
      const int i = j + 1 + e / w, l = j + 1 + e % w;
      if (l >= i) A[i * LD + l] -= A[j * LD + i] * A[j * LD + l];
    }
    __syncthreads();
  }
  __syncthreads();
  if (bad) {
    if (tid == 0) *info = bad;
    return;
  }
  // R^-1 column by column (back substitution), one thread per column
  for (int c = tid; c < M; c += SVQB_THREADS) {
    for (int i = M - 1; i >= 0; i--) {
      double v = (i == c) ? 1.0 : 0.0;
      for (int k = i + 1; k <= c; k++) v -= A[i * LD + k] * Y[k * LD + c];
      Y[i * LD + c] = i > c ? 0.0 : v / A[i * LD + i];
    }
  }
  __syncthreads();
  for (int e = tid; e < M * M; e += SVQB_THREADS) {
    const int n = e / M, m = e % M;
    T[e] = Y[m * LD + n];
  }
  if (tid == 0) *info = 0;
}

static size_t svqb_eig_smem(int M) {
  return (size_t)(2 * M * (M + 1) + M + 2 * (M / 2 + 1) + SVQB_THREADS) * sizeof(double) +
         (SVQB_MAX_M + 2 * (M / 2 + 1)) * sizeof(int) + 64;
}

}  // namespace skinny

using namespace skinny;

extern "C" skinny_status skinny_svqb(skinny_handle h, skinny_acc gram_acc, int64_t K, int64_t M,
                                     double* X, int64_t ldx, double* orth_err_out, void* stream) {
  set_error("");
  if (!h) {
    set_error("null handle");
    return SKINNY_BAD_ARG;
  }
  if (M < 1 || K < 0 || ldx < M || (K > 0 && !X)) {
    set_error("svqb: bad sizes or null X");
    return SKINNY_BAD_ARG;
  }
  if (M > SVQB_MAX_M) {
    set_error("svqb: M > 64 not provided");
    return SKINNY_UNSUPPORTED;
  }
  DevGuard g(h->dev.id);
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(h->mu);
  // scratch: S, T, S2 (M x M each) + error word + sweep count
  const size_t need = (3 * (size_t)SVQB_MAX_M * SVQB_MAX_M + 8) * sizeof(double);
  void*& buf = h->svqb_ws[st];
  if (!buf) {
    if (cudaMalloc(&buf, need) != cudaSuccess) {
      cudaGetLastError();
      buf = nullptr;
      set_error("svqb: cudaMalloc failed");
      return SKINNY_NO_MEM;
    }
    h->extra_allocs.push_back(buf);
  }
  double* S = static_cast<double*>(buf);
  double* T = S + SVQB_MAX_M * SVQB_MAX_M;
  double* S2 = T + SVQB_MAX_M * SVQB_MAX_M;
  double* errd = S2 + SVQB_MAX_M * SVQB_MAX_M;
  int* info = reinterpret_cast<int*>(errd + 1);
  const double one = 1.0, zero = 0.0;
  LaunchOpts o{};
  skinny_status s = dispatch_product(h, false, SKINNY_R64, gram_acc, M, M, K, X, ldx, &one, X, ldx,
                                     &zero, S, M, st, o);
  if (s == SKINNY_UNSUPPORTED && gram_acc == SKINNY_ACC_SPLIT)  // split not provided at this M
    s = dispatch_product(h, false, SKINNY_R64, SKINNY_ACC_NATIVE, M, M, K, X, ldx, &one, X, ldx, &zero, S,
                         M, st, o);
  if (s != SKINNY_OK) return s;
  const size_t smem = svqb_eig_smem((int)M);
  static SmemAttr attr;
  ensure_smem_attr(svqb_eig_kernel, (int)smem, attr);
  svqb_eig_kernel<<<1, SVQB_THREADS, smem, st>>>(S, (int)M, T, info, 30);
  count_launch();
  if (cudaGetLastError() != cudaSuccess) {
    set_error("svqb: eigensolver launch failed");
    return SKINNY_DEVICE_ERROR;
  }
  s = dispatch_product(h, true, SKINNY_R64, SKINNY_ACC_AUTO, M, M, K, X, ldx, &one, T, M, &zero, X,
                       ldx, st, o);
  if (s != SKINNY_OK) return s;
  if (orth_err_out) {
    s = dispatch_product(h, false, SKINNY_R64, SKINNY_ACC_DD, M, M, K, X, ldx, &one, X, ldx, &zero, S2,
                         M, st, o);
    if (s != SKINNY_OK) return s;
    svqb_orth_kernel<<<1, SVQB_THREADS, 0, st>>>(S2, (int)M, errd);
    count_launch();
    double v = -1.0;
    if (cudaMemcpyAsync(&v, errd, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cudaGetLastError();
      set_error("svqb: reading the orthogonality error failed");
      return SKINNY_DEVICE_ERROR;
    }
    *orth_err_out = v;
  }
  return SKINNY_OK;
}

// CholQR (passes = 1) / CholQR2 (passes = 2): Gram, Cholesky and in-place TSMM with R^-1 per pass.
// No counterpart in the reference (whose orthogonalisation is SVQB, svqb/svqb.cu:72-130); it
// reuses the same Gram and in-place TSMM.  SKINNY_BAD_ARG when a Gram is not numerically positive
// definite (X is then left as the previous pass made it).
extern "C" skinny_status skinny_cholqr(skinny_handle h, skinny_acc gram_acc, int64_t K, int64_t M, double* X,
                                       int64_t ldx, int passes, double* orth_err_out, void* stream) {
  set_error("");
  if (!h) {
    set_error("null handle");
    return SKINNY_BAD_ARG;
  }
  if (M < 1 || K < 0 || ldx < M || (K > 0 && !X) || passes < 1 || passes > 4) {
    set_error("cholqr: bad sizes, null X or passes outside 1..4");
    return SKINNY_BAD_ARG;
  }
  if (M > SVQB_MAX_M) {
    set_error("cholqr: M > 64 not provided");
    return SKINNY_UNSUPPORTED;
  }
  DevGuard g(h->dev.id);
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(h->mu);
  const size_t need = (3 * (size_t)SVQB_MAX_M * SVQB_MAX_M + 8) * sizeof(double);
  void*& buf = h->svqb_ws[st];
  if (!buf) {
    if (cudaMalloc(&buf, need) != cudaSuccess) {
      cudaGetLastError();
      buf = nullptr;
      set_error("cholqr: cudaMalloc failed");
      return SKINNY_NO_MEM;
    }
    h->extra_allocs.push_back(buf);
  }
  double* S = static_cast<double*>(buf);
  double* T = S + SVQB_MAX_M * SVQB_MAX_M;
  double* S2 = T + SVQB_MAX_M * SVQB_MAX_M;
  double* errd = S2 + SVQB_MAX_M * SVQB_MAX_M;
  int* info = reinterpret_cast<int*>(errd + 1);
  const double one = 1.0, zero = 0.0;
  LaunchOpts o{};
  const size_t smem = (size_t)2 * M * (M + 1) * sizeof(double);
  static SmemAttr attr;
  ensure_smem_attr(cholqr_kernel, (int)smem, attr);
  for (int pass = 0; pass < passes; pass++) {
    skinny_status s = dispatch_product(h, false, SKINNY_R64, gram_acc, M, M, K, X, ldx, &one, X, ldx, &zero, S, M,
                                       st, o);
    if (s == SKINNY_UNSUPPORTED && gram_acc == SKINNY_ACC_SPLIT)
      s = dispatch_product(h, false, SKINNY_R64, SKINNY_ACC_NATIVE, M, M, K, X, ldx, &one, X, ldx, &zero, S, M, st, o);
    if (s != SKINNY_OK) return s;
    cholqr_kernel<<<1, SVQB_THREADS, smem, st>>>(S, (int)M, T, info);
    count_launch();
    int hinfo = 0;
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cudaGetLastError();
      set_error("cholqr: Cholesky launch failed");
      return SKINNY_DEVICE_ERROR;
    }
    if (hinfo != 0) {
      set_error("cholqr: Gram matrix not positive definite at column " + std::to_string(hinfo - 1));
      return SKINNY_BAD_ARG;
    }
    s = dispatch_product(h, true, SKINNY_R64, SKINNY_ACC_AUTO, M, M, K, X, ldx, &one, T, M, &zero, X, ldx, st, o);
    if (s != SKINNY_OK) return s;
  }
  if (orth_err_out) {
    skinny_status s = dispatch_product(h, false, SKINNY_R64, SKINNY_ACC_DD, M, M, K, X, ldx, &one, X, ldx, &zero,
                                       S2, M, st, o);
    if (s != SKINNY_OK) return s;
    svqb_orth_kernel<<<1, SVQB_THREADS, 0, st>>>(S2, (int)M, errd);
    count_launch();
    double v = -1.0;
    if (cudaMemcpyAsync(&v, errd, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cudaGetLastError();
      set_error("cholqr: reading the orthogonality error failed");
      return SKINNY_DEVICE_ERROR;
    }
    *orth_err_out = v;
  }
  return SKINNY_OK;
}
