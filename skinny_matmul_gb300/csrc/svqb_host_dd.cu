// svqb_host_dd.cu -- SVQB in double-double on the host (the reference's high-precision study,
// svqb/svqb.cu:132-182 svqb_xd<dd_real>, which calls MPACK's Rgemm / Rsyev).  Host code only:
// the accuracy baseline for the device SVQB (svqb.cu) at high condition numbers, where a
// one-pass FP64 SVQB loses orthogonality as kappa^2 u.
//
// Steps as in the reference, every one in double-double:
//   S = X^T X; d_i = 1/sqrt(S_ii) (0 when S_ii <= eps, eps the double-double epsilon 2^-104);
//   S <- D S D; S = U diag(l) U^T (cyclic Jacobi; the reference calls Rsyev); columns of U in
//   ascending order of l, each with its largest entry positive;
//   T[n][m] = U[m][n] d_m / sqrt(l_n) (d_m when |l_n| <= eps); Q = X T^T, rounded to double.
// The double-double arithmetic is written here from the error-free transformations (Knuth's
// two-sum, Dekker's fast two-sum, the FMA two-product) with Newton steps for division and square
// root; Gram and Q = X T^T run on host threads over row ranges (partials summed in a fixed order).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "api_internal.h"

namespace skinny {
namespace hostdd {

struct D2 {
  double hi, lo;
};
inline D2 two_sum(double a, double b) {
  const double s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
inline D2 fast_two_sum(double a, double b) {  // |a| >= |b| or a == 0
  const double s = a + b;
  return {s, b - (s - a)};
}
inline D2 two_prod(double a, double b) {
  const double p = a * b;
  return {p, std::fma(a, b, -p)};
}
inline D2 add(D2 a, D2 b) {
  D2 s = two_sum(a.hi, b.hi);
  const D2 t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
inline D2 neg(D2 a) { return {-a.hi, -a.lo}; }
inline D2 sub(D2 a, D2 b) { return add(a, neg(b)); }
inline D2 mul(D2 a, D2 b) {
  D2 p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return fast_two_sum(p.hi, p.lo);
}
inline D2 mul(D2 a, double b) {
  D2 p = two_prod(a.hi, b);
  p.lo += a.lo * b;
  return fast_two_sum(p.hi, p.lo);
}
// exact product of two doubles added to a double-double
inline D2 mac(D2 acc, double a, double b) { return add(acc, two_prod(a, b)); }
inline D2 div(D2 a, D2 b) {  // three quotient digits, each from the remainder
  const double q1 = a.hi / b.hi;
  D2 r = sub(a, mul(b, q1));
  const double q2 = r.hi / b.hi;
  r = sub(r, mul(b, q2));
  const double q3 = r.hi / b.hi;
  return add(fast_two_sum(q1, q2), D2{q3, 0.0});
}
inline D2 sqrt(D2 a) {  // one Newton step from the double square root: x + (a - x^2) / (2x)
  if (a.hi <= 0.0) return {0.0, 0.0};
  const double x = std::sqrt(a.hi);
  const D2 r = sub(a, two_prod(x, x));
  return fast_two_sum(x, r.hi / (2.0 * x));
}
inline double absd(D2 a) { return std::fabs(a.hi); }
inline bool lt(D2 a, D2 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
inline double to_double(D2 a) { return a.hi + a.lo; }
constexpr double EPS = 4.93038065763132e-32;  // 2^-104

// Gram S[m][n] (m <= n) over rows [k0, k1)
void gram_rows(const double* X, int M, int64_t k0, int64_t k1, D2* S) {
  for (int i = 0; i < M * M; i++) S[i] = {0.0, 0.0};
  for (int64_t k = k0; k < k1; k++) {
    const double* x = X + k * M;
    for (int m = 0; m < M; m++)
      for (int n = m; n < M; n++) S[m * M + n] = mac(S[m * M + n], x[m], x[n]);
  }
}

template <class F>
void parallel_rows(int64_t K, int threads, F&& f) {
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) {
    const int64_t k0 = K * t / threads, k1 = K * (t + 1) / threads;
    pool.emplace_back([=, &f] { f(t, k0, k1); });
  }
  for (auto& th : pool) th.join();
}

// cyclic Jacobi on the symmetric A (M x M, full storage); V gets the eigenvectors as columns
void jacobi(std::vector<D2>& A, std::vector<D2>& V, int M) {
  for (int i = 0; i < M; i++)
    for (int j = 0; j < M; j++) V[i * M + j] = {i == j ? 1.0 : 0.0, 0.0};
  double prev = INFINITY;
  for (int sweep = 0; sweep < 60; sweep++) {
    D2 off = {0.0, 0.0}, tot = {0.0, 0.0};
    for (int i = 0; i < M; i++)
      for (int j = 0; j < M; j++) {
        const D2 s = mul(A[i * M + j], A[i * M + j]);
        tot = add(tot, s);
        if (i != j) off = add(off, s);
      }
    // converged: the off-diagonal mass is at the double-double rounding of the matrix, or has
    // stopped shrinking
    if (off.hi <= EPS * EPS * tot.hi || !(off.hi < prev)) break;
    prev = off.hi;
    for (int p = 0; p < M - 1; p++)
      for (int q = p + 1; q < M; q++) {
        const D2 apq = A[p * M + q];
        if (absd(apq) == 0.0) continue;
        // theta = (a_qq - a_pp) / (2 a_pq); t = sign(theta) / (|theta| + sqrt(theta^2 + 1))
        const D2 theta = div(sub(A[q * M + q], A[p * M + p]), mul(apq, 2.0));
        const D2 at = theta.hi < 0 ? neg(theta) : theta;
        D2 t = div(D2{1.0, 0.0}, add(at, sqrt(add(mul(theta, theta), D2{1.0, 0.0}))));
        if (theta.hi < 0) t = neg(t);
        const D2 c = div(D2{1.0, 0.0}, sqrt(add(mul(t, t), D2{1.0, 0.0})));
        const D2 s = mul(t, c);
        for (int k = 0; k < M; k++) {  // columns p, q
          const D2 akp = A[k * M + p], akq = A[k * M + q];
          A[k * M + p] = sub(mul(c, akp), mul(s, akq));
          A[k * M + q] = add(mul(s, akp), mul(c, akq));
        }
        for (int k = 0; k < M; k++) {  // rows p, q
          const D2 apk = A[p * M + k], aqk = A[q * M + k];
          A[p * M + k] = sub(mul(c, apk), mul(s, aqk));
          A[q * M + k] = add(mul(s, apk), mul(c, aqk));
        }
        for (int k = 0; k < M; k++) {
          const D2 vkp = V[k * M + p], vkq = V[k * M + q];
          V[k * M + p] = sub(mul(c, vkp), mul(s, vkq));
          V[k * M + q] = add(mul(s, vkp), mul(c, vkq));
        }
      }
  }
}

}  // namespace hostdd
}  // namespace skinny

using namespace skinny::hostdd;

extern "C" skinny_status skinny_svqb_host_dd(const double* X, double* Q, int64_t K, int M, int threads,
                                             double* orth_err_out) {
  skinny::set_error("");
  if (!X || !Q || K < 0 || M < 1 || M > 256) {
    skinny::set_error("svqb_host_dd: null array, K < 0 or M outside 1..256");
    return SKINNY_BAD_ARG;
  }
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  threads = (int)std::max<int64_t>(1, std::min<int64_t>(threads, std::max<int64_t>(1, K / 64)));
  // S = X^T X: per-thread partials over row ranges, summed in thread order
  std::vector<std::vector<D2>> part(threads, std::vector<D2>((size_t)M * M));
  parallel_rows(K, threads, [&](int t, int64_t k0, int64_t k1) { gram_rows(X, M, k0, k1, part[t].data()); });
  std::vector<D2> S((size_t)M * M, D2{0.0, 0.0});
  for (int t = 0; t < threads; t++)
    for (int i = 0; i < M * M; i++) S[i] = add(S[i], part[t][i]);
  for (int m = 0; m < M; m++)
    for (int n = 0; n < m; n++) S[m * M + n] = S[n * M + m];
  // D^-1/2 scaling
  std::vector<D2> dinv(M);
  for (int i = 0; i < M; i++)
    dinv[i] = S[i * M + i].hi > EPS ? div(D2{1.0, 0.0}, sqrt(S[i * M + i])) : D2{0.0, 0.0};
  for (int m = 0; m < M; m++)
    for (int n = 0; n < M; n++) S[m * M + n] = mul(S[m * M + n], mul(dinv[m], dinv[n]));
  // eigensolve, ascending eigenvalues, each vector's largest entry positive
  std::vector<D2> V((size_t)M * M);
  jacobi(S, V, M);
  std::vector<int> order(M);
  for (int i = 0; i < M; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return lt(S[a * M + a], S[b * M + b]); });
  // T[n][m] = U[m][n] d_m / sqrt(l_n), or d_m when |l_n| <= eps
  std::vector<D2> T((size_t)M * M);
  for (int n = 0; n < M; n++) {
    const int j = order[n];
    int big = 0;
    for (int m = 1; m < M; m++)
      if (absd(V[m * M + j]) > absd(V[big * M + j])) big = m;
    const bool flip = V[big * M + j].hi < 0;
    const D2 l = S[j * M + j];
    const bool tiny = absd(l) <= EPS;
    const D2 isl = tiny ? D2{1.0, 0.0} : div(D2{1.0, 0.0}, sqrt(l));
    for (int m = 0; m < M; m++) {
      const D2 u = flip ? neg(V[m * M + j]) : V[m * M + j];
      T[n * M + m] = tiny ? dinv[m] : mul(mul(u, dinv[m]), isl);
    }
  }
  // Q = X T^T, rounded to double once
  parallel_rows(K, threads, [&](int, int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; k++) {
      const double* x = X + k * M;
      for (int n = 0; n < M; n++) {
        D2 acc = {0.0, 0.0};
        for (int m = 0; m < M; m++) {
          const D2 p = mul(T[n * M + m], x[m]);
          acc = add(acc, p);
        }
        Q[k * M + n] = to_double(acc);
      }
    }
  });
  if (orth_err_out) {  // ||Q^T Q - I||_F of the rounded Q, Gram in double-double
    parallel_rows(K, threads, [&](int t, int64_t k0, int64_t k1) { gram_rows(Q, M, k0, k1, part[t].data()); });
    D2 e2 = {0.0, 0.0};
    for (int m = 0; m < M; m++)
      for (int n = m; n < M; n++) {
        D2 s = {0.0, 0.0};
        for (int t = 0; t < threads; t++) s = add(s, part[t][m * M + n]);
        if (m == n) s = sub(s, D2{1.0, 0.0});
        const D2 s2 = mul(s, s);
        e2 = add(e2, m == n ? s2 : mul(s2, 2.0));
      }
    *orth_err_out = to_double(sqrt(e2));
  }
  return SKINNY_OK;
}
