// svqb_complex.cu -- SVQB of a complex FP64 block on the device (no counterpart in the reference,
// whose SVQB is real, svqb/svqb.cu:72-130): the same steps with the Hermitian Gram S = X^H X
// (skinny_tsmttsm_conj), a Hermitian Jacobi eigensolve and the complex in-place TSMM.
//
// Hermitian Jacobi: for a pair (p, q) with a_pq = |a_pq| e^{-i phi}, the unitary
// U = diag(1, e^{i phi}) [[c, s], [-s, c]] makes the pivot block real and then zeroes it as the
// real rotation does (c, s from the real 2x2 block [[a_pp, |a_pq|], [|a_pq|, a_qq]]):
//   columns (A U, V U):  p <- c p - s w q,        q <- s p + c w q        (w = e^{i phi})
//   rows (U^H A):        p <- c p - s conj(w) q,  q <- s p + c conj(w) q
// Round-robin pairs as in svqb.cu; eigenvalues ascending; each eigenvector's largest-magnitude
// entry made real and positive.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>

#include "api_internal.h"

namespace skinny {

namespace {

constexpr int CMAXM = 64;
constexpr int CTHREADS = 256;

struct z2 {
  double x, y;
};
__device__ __forceinline__ z2 zmul(z2 a, z2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ z2 zconj(z2 a) { return {a.x, -a.y}; }

__global__ void __launch_bounds__(CTHREADS) svqbz_eig_kernel(const z2* __restrict__ S, int M, z2* __restrict__ T,
                                                             int max_sweeps) {
  extern __shared__ __align__(16) unsigned char raw[];
  const int LD = M + 1;
  z2* A = reinterpret_cast<z2*>(raw);  // M x LD
  z2* V = A + M * LD;                  // M x LD
  double* d = reinterpret_cast<double*>(V + M * LD);  // M
  double* cs = d + M;                                  // [npairs][4]: c, s, w.x, w.y
  double* red = cs + 4 * (CMAXM / 2 + 1);              // CTHREADS
  int* pq = reinterpret_cast<int*>(red + CTHREADS);    // [npairs][2]
  int* order = pq + 2 * (CMAXM / 2 + 1);               // M
  const int tid = threadIdx.x;
  constexpr int KS = CTHREADS / CMAXM;
  const int i0 = tid % CMAXM, k0 = tid / CMAXM;

  for (int i = tid; i < M; i += CTHREADS) {
    const double sii = S[i * M + i].x;
    d[i] = fabs(sii) > 1.0e-15 ? 1.0 / sqrt(sii) : 0.0;
  }
  __syncthreads();
  for (int e = tid; e < M * M; e += CTHREADS) {  // S[n*M + m] = sum conj(x_m) x_n: row m, column n
    const int n = e / M, m = e % M;
    const z2 v = S[e];
    A[m * LD + n] = {v.x * d[m] * d[n], v.y * d[m] * d[n]};
    V[m * LD + n] = {m == n ? 1.0 : 0.0, 0.0};
  }
  __syncthreads();

  const int np = (M + 1) & ~1, npairs = np / 2;
  const double tol = (double)M * M * 1.23e-32;
  double prev_off = 0.0;
  for (int sweep = 0; sweep < max_sweeps; sweep++) {
    double off = 0.0, all = 0.0;
    for (int e = tid; e < M * M; e += CTHREADS) {
      const int i = e / M, j = e % M;
      const z2 a = A[i * LD + j];
      const double a2 = a.x * a.x + a.y * a.y;
      all += a2;
      if (i != j) off += a2;
    }
    red[tid] = off;
    __syncthreads();
    for (int s = CTHREADS / 2; s > 0; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    const double off_sum = red[0];
    __syncthreads();
    red[tid] = all;
    __syncthreads();
    for (int s = CTHREADS / 2; s > 0; s >>= 1) {
      if (tid < s) red[tid] += red[tid + s];
      __syncthreads();
    }
    const double all_sum = red[0];
    __syncthreads();
    if (off_sum <= tol * all_sum || M == 1 || (sweep > 0 && off_sum <= 1.0e-20 * all_sum && off_sum >= 0.25 * prev_off))
      break;
    prev_off = off_sum;

    for (int r = 0; r < np - 1; r++) {
      for (int k = tid; k < npairs; k += CTHREADS) {
        int p = k == 0 ? np - 1 : (r + k) % (np - 1);
        int q = k == 0 ? r : (r - k + np - 1) % (np - 1);
        if (p > q) {
          const int x = p;
          p = q;
          q = x;
        }
        double c = 1.0, s = 0.0, wx = 1.0, wy = 0.0;
        if (q < M) {
          const z2 apq = A[p * LD + q];
          const double mag = hypot(apq.x, apq.y);
          if (mag != 0.0) {
            wx = apq.x / mag;  // w = conj(a_pq / |a_pq|): a_pq w = |a_pq|
            wy = -apq.y / mag;
            const double tau = (A[q * LD + q].x - A[p * LD + p].x) / (2.0 * mag);
            const double t = tau >= 0.0 ? 1.0 / (tau + sqrt(1.0 + tau * tau)) : -1.0 / (-tau + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        } else {
          q = p;
        }
        cs[4 * k] = c;
        cs[4 * k + 1] = s;
        cs[4 * k + 2] = wx;
        cs[4 * k + 3] = wy;
        pq[2 * k] = p;
        pq[2 * k + 1] = q;
      }
      __syncthreads();
      if (i0 < M)  // columns: A U and V U, row i0
        for (int k = k0; k < npairs; k += KS) {
          const int p = pq[2 * k], q = pq[2 * k + 1];
          if (p == q) continue;
          const double c = cs[4 * k], s = cs[4 * k + 1];
          const z2 w = {cs[4 * k + 2], cs[4 * k + 3]};
          const z2 ap = A[i0 * LD + p], aq = zmul(w, A[i0 * LD + q]);
          A[i0 * LD + p] = {c * ap.x - s * aq.x, c * ap.y - s * aq.y};
          A[i0 * LD + q] = {s * ap.x + c * aq.x, s * ap.y + c * aq.y};
          const z2 vp = V[i0 * LD + p], vq = zmul(w, V[i0 * LD + q]);
          V[i0 * LD + p] = {c * vp.x - s * vq.x, c * vp.y - s * vq.y};
          V[i0 * LD + q] = {s * vp.x + c * vq.x, s * vp.y + c * vq.y};
        }
      __syncthreads();
      if (i0 < M)  // rows: U^H A, column i0
        for (int k = k0; k < npairs; k += KS) {
          const int p = pq[2 * k], q = pq[2 * k + 1];
          if (p == q) continue;
          const double c = cs[4 * k], s = cs[4 * k + 1];
          const z2 wc = zconj({cs[4 * k + 2], cs[4 * k + 3]});
          const z2 ap = A[p * LD + i0], aq = zmul(wc, A[q * LD + i0]);
          A[p * LD + i0] = {c * ap.x - s * aq.x, c * ap.y - s * aq.y};
          A[q * LD + i0] = {s * ap.x + c * aq.x, s * ap.y + c * aq.y};
        }
      __syncthreads();
    }
  }

  for (int i = tid; i < M; i += CTHREADS) {
    const double li = A[i * LD + i].x;
    int rank = 0;
    for (int j = 0; j < M; j++) {
      const double lj = A[j * LD + j].x;
      rank += (lj < li) || (lj == li && j < i);
    }
    order[rank] = i;
  }
  __syncthreads();
  // T[col*M + m] = V[m][src] * phase * d[m] / sqrt(max(1e-15, l_src)), phase making the largest
  // |V[.][src]| real positive
  for (int col = tid; col < M; col += CTHREADS) {
    const int src = order[col];
    double big = -1.0;
    z2 ph = {1.0, 0.0};
    for (int m = 0; m < M; m++) {
      const z2 v = V[m * LD + src];
      const double a = hypot(v.x, v.y);
      if (a > big) {
        big = a;
        ph = a > 0.0 ? z2{v.x / a, -v.y / a} : z2{1.0, 0.0};
      }
    }
    const double f = 1.0 / sqrt(fmax(1.0e-15, A[src * LD + src].x));
    for (int m = 0; m < M; m++) {
      const z2 v = zmul(V[m * LD + src], ph);
      T[col * M + m] = {v.x * d[m] * f, v.y * d[m] * f};
    }
  }
}

// ||S - I||_F for a complex M x M matrix
__global__ void __launch_bounds__(CTHREADS) svqbz_orth_kernel(const z2* __restrict__ S, int M, double* out) {
  __shared__ double red[CTHREADS];
  double acc = 0.0;
  for (int e = threadIdx.x; e < M * M; e += CTHREADS) {
    const z2 v = S[e];
    const double re = v.x - ((e / M == e % M) ? 1.0 : 0.0);
    acc += re * re + v.y * v.y;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = CTHREADS / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sqrt(red[0]);
}

size_t eig_smem(int M) {
  return (size_t)2 * M * (M + 1) * sizeof(z2) + (M + 4 * (CMAXM / 2 + 1) + CTHREADS) * sizeof(double) +
         (2 * (CMAXM / 2 + 1) + CMAXM) * sizeof(int) + 64;
}

}  // namespace

}  // namespace skinny

using namespace skinny;

extern "C" skinny_status skinny_svqb_z(skinny_handle h, skinny_acc gram_acc, int64_t K, int64_t M, void* X,
                                       int64_t ldx, double* orth_err_out, void* stream) {
  set_error("");
  if (!h) {
    set_error("null handle");
    return SKINNY_BAD_ARG;
  }
  if (M < 1 || K < 0 || ldx < M || (K > 0 && !X)) {
    set_error("svqb_z: bad sizes or null X");
    return SKINNY_BAD_ARG;
  }
  if (M > CMAXM) {
    set_error("svqb_z: M > 64 not provided");
    return SKINNY_UNSUPPORTED;
  }
  DevGuard g(h->dev.id);
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(h->mu);
  // scratch after the real SVQB's (S, T, S2 complex, M x M each) in its own per-stream block
  void*& buf = h->svqbz_ws[st];
  if (!buf) {
    if (cudaMalloc(&buf, (3 * (size_t)CMAXM * CMAXM + 4) * sizeof(z2)) != cudaSuccess) {
      cudaGetLastError();
      buf = nullptr;
      set_error("svqb_z: cudaMalloc failed");
      return SKINNY_NO_MEM;
    }
    h->extra_allocs.push_back(buf);
  }
  z2* S = static_cast<z2*>(buf);
  z2* T = S + CMAXM * CMAXM;
  z2* S2 = T + CMAXM * CMAXM;
  double* errd = reinterpret_cast<double*>(S2 + CMAXM * CMAXM);
  const double one[2] = {1.0, 0.0}, zero[2] = {0.0, 0.0};
  skinny_status s = dispatch_conj(h, SKINNY_C64, gram_acc, M, M, K, X, ldx, one, X, ldx, zero, S, M, st);
  if (s == SKINNY_UNSUPPORTED && gram_acc == SKINNY_ACC_SPLIT)
    s = dispatch_conj(h, SKINNY_C64, SKINNY_ACC_NATIVE, M, M, K, X, ldx, one, X, ldx, zero, S, M, st);
  if (s != SKINNY_OK) return s;
  const size_t smem = eig_smem((int)M);
  static SmemAttr attr;
  ensure_smem_attr(svqbz_eig_kernel, (int)smem, attr);
  svqbz_eig_kernel<<<1, CTHREADS, smem, st>>>(S, (int)M, T, 30);
  count_launch();
  if (cudaGetLastError() != cudaSuccess) {
    set_error("svqb_z: eigensolver launch failed");
    return SKINNY_DEVICE_ERROR;
  }
  LaunchOpts o{};
  s = dispatch_product(h, true, SKINNY_C64, SKINNY_ACC_AUTO, M, M, K, X, ldx, one, T, M, zero, X, ldx, st, o);
  if (s != SKINNY_OK) return s;
  if (orth_err_out) {
    s = dispatch_conj(h, SKINNY_C64, SKINNY_ACC_AUTO, M, M, K, X, ldx, one, X, ldx, zero, S2, M, st);
    if (s != SKINNY_OK) return s;
    svqbz_orth_kernel<<<1, CTHREADS, 0, st>>>(S2, (int)M, errd);
    count_launch();
    double v = -1.0;
    if (cudaMemcpyAsync(&v, errd, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      cudaGetLastError();
      set_error("svqb_z: reading the orthogonality error failed");
      return SKINNY_DEVICE_ERROR;
    }
    *orth_err_out = v;
  }
  return SKINNY_OK;
}
