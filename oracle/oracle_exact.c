/* oracle_exact.c -- exact super-accumulator and double-double ("PseudoQuad") restatement.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Compiled with -ffp-contract=off so every
 * multiply and add below rounds exactly as written; fma() is only used where the reference's
 * PseudoQuad.cuh uses __fma_rn.
 *
 * The super-accumulator is a fixed-point integer of 72 signed 32-bit limbs held in int64
 * (carry-save), covering bit weights 2^-1152 .. 2^1152.  Every finite double product of
 * moderate operands is added exactly (two-product split through fma), so the accumulated
 * value is the exact real sum; it is then rounded once to double (hi) and the exact remainder
 * rounded once more (lo).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"

#define XA_LIMBS 72
#define XA_BASE (-1152) /* weight of bit 0 of limb 0 */

typedef struct {
  int64_t l[XA_LIMBS];
  int64_t pending;
} xacc;

static void xa_init(xacc* a) { memset(a, 0, sizeof(*a)); }

static void xa_norm(xacc* a) {
  for (int i = 0; i < XA_LIMBS - 1; i++) {
    int64_t c = a->l[i] >> 32; /* arithmetic shift: floor division */
    a->l[i] -= c * ((int64_t)1 << 32);
    a->l[i + 1] += c;
  }
  a->pending = 0;
}

static void xa_add(xacc* a, double x) {
  if (x == 0.0) return;
  int e;
  double f = frexp(x, &e);                   /* x = f * 2^e, 0.5 <= |f| < 1 */
  int64_t mant = (int64_t)ldexp(f, 53);      /* exact, |mant| < 2^53 */
  int p = e - 53 - XA_BASE;                  /* weight of mant's lowest bit */
  int i = p >> 5, s = p & 31;
  uint64_t m = (uint64_t)(mant < 0 ? -mant : mant);
  unsigned __int128 v = (unsigned __int128)m << s;
  int64_t l0 = (int64_t)(uint32_t)v;
  int64_t l1 = (int64_t)(uint32_t)(v >> 32);
  int64_t l2 = (int64_t)(uint32_t)(v >> 64);
  if (mant < 0) {
    a->l[i] -= l0; a->l[i + 1] -= l1; a->l[i + 2] -= l2;
  } else {
    a->l[i] += l0; a->l[i + 1] += l1; a->l[i + 2] += l2;
  }
  if (++a->pending >= ((int64_t)1 << 28)) xa_norm(a);
}

/* exact a*b (no underflow/overflow assumed for the operands used in tests) */
static void xa_add_prod(xacc* a, double x, double y) {
  double p = x * y;
  double e = fma(x, y, -p);
  xa_add(a, p);
  xa_add(a, e);
}

/* round the exact value to the nearest double (ties to even); subnormal results not handled */
static double xa_round(const xacc* in) {
  xacc a = *in;
  xa_norm(&a);
  int neg = a.l[XA_LIMBS - 1] < 0;
  if (neg) {
    for (int i = 0; i < XA_LIMBS; i++) a.l[i] = -a.l[i];
    xa_norm(&a);
  }
  int top = -1;
  for (int i = XA_LIMBS - 1; i >= 0; i--)
    if (a.l[i] != 0) { top = i; break; }
  if (top < 0) return 0.0;
  int hb = 63 - __builtin_clzll((unsigned long long)a.l[top]);
  int P = top * 32 + hb; /* absolute position of the leading one */
  /* gather bits [P-63, P] into u64 and a sticky flag below */
  uint64_t bits = 0;
  for (int k = 0; k < 64; k++) {
    int q = P - k;
    uint64_t b = 0;
    if (q >= 0) b = ((uint64_t)a.l[q >> 5] >> (q & 31)) & 1u;
    bits = (bits << 1) | b;
  }
  int sticky = 0;
  int lk = P - 63; /* lowest gathered position; sticky = any one bit below it */
  if (lk > 0) {
    int j = lk >> 5;
    uint64_t below = (uint64_t)a.l[j] & ((((uint64_t)1) << (lk & 31)) - 1u);
    if (below) sticky = 1;
    for (int i = 0; i < j && !sticky; i++)
      if (a.l[i] != 0) sticky = 1;
  }
  uint64_t mant = bits >> 11;
  uint64_t rem = bits & 0x7FFu;
  if (rem > 0x400u || (rem == 0x400u && (sticky || (mant & 1u)))) mant++;
  double r = ldexp((double)mant, P - 52 + XA_BASE);
  return neg ? -r : r;
}

static void xa_round_dd(xacc* a, double* hi, double* lo) {
  double h = xa_round(a);
  xa_add(a, -h);
  double l = xa_round(a);
  xa_add(a, h); /* restore */
  *hi = h;
  *lo = l;
}

static int nthr(int n) {
#ifdef _OPENMP
  return n > 0 ? n : omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int orc_max_threads(void) { return nthr(0); }

void orc_dot_exact(int64_t K, const double* a, int64_t inca, const double* b, int64_t incb,
                   double* hi, double* lo) {
  xacc x;
  xa_init(&x);
  for (int64_t k = 0; k < K; k++) xa_add_prod(&x, a[k * inca], b[k * incb]);
  xa_round_dd(&x, hi, lo);
}

/* ---- TSMTTSM exact: S[n*lds+m] = sum_k A[k*lda+m] B[k*ldb+n] ---------------------------- */
void orc_tsmttsm_exact_d(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                         const double* B, int64_t ldb, double* hi, double* lo, int64_t lds,
                         int nthreads) {
  int64_t MN = M * N;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthr(nthreads))
  for (int64_t mn = 0; mn < MN; mn++) {
    int64_t m = mn % M, n = mn / M;
    xacc x;
    xa_init(&x);
    for (int64_t k = 0; k < K; k++) xa_add_prod(&x, A[k * lda + m], B[k * ldb + n]);
    xa_round_dd(&x, &hi[n * lds + m], &lo[n * lds + m]);
  }
}

void orc_tsmttsm_exact_z(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                         const double* B, int64_t ldb, double* hi, double* lo, int64_t lds,
                         int nthreads) {
  int64_t MN = M * N;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthr(nthreads))
  for (int64_t mn = 0; mn < MN; mn++) {
    int64_t m = mn % M, n = mn / M;
    xacc re, im;
    xa_init(&re);
    xa_init(&im);
    for (int64_t k = 0; k < K; k++) {
      double ar = A[2 * (k * lda + m)], ai = A[2 * (k * lda + m) + 1];
      double br = B[2 * (k * ldb + n)], bi = B[2 * (k * ldb + n) + 1];
      xa_add_prod(&re, ar, br);
      xa_add_prod(&re, -ai, bi);
      xa_add_prod(&im, ar, bi);
      xa_add_prod(&im, ai, br);
    }
    int64_t o = 2 * (n * lds + m);
    xa_round_dd(&re, &hi[o], &lo[o]);
    xa_round_dd(&im, &hi[o + 1], &lo[o + 1]);
  }
}

/* ---- TSMM exact: S[r*lds+n] = sum_m A[r*lda+m] B[n*ldb+m] -------------------------------- */
void orc_tsmm_exact_d(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                      const double* B, int64_t ldb, double* hi, double* lo, int64_t lds,
                      int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthr(nthreads))
  for (int64_t r = 0; r < K; r++) {
    for (int64_t n = 0; n < N; n++) {
      xacc x;
      xa_init(&x);
      for (int64_t m = 0; m < M; m++) xa_add_prod(&x, A[r * lda + m], B[n * ldb + m]);
      xa_round_dd(&x, &hi[r * lds + n], &lo[r * lds + n]);
    }
  }
}

void orc_tsmm_exact_z(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda,
                      const double* B, int64_t ldb, double* hi, double* lo, int64_t lds,
                      int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthr(nthreads))
  for (int64_t r = 0; r < K; r++) {
    for (int64_t n = 0; n < N; n++) {
      xacc re, im;
      xa_init(&re);
      xa_init(&im);
      for (int64_t m = 0; m < M; m++) {
        double ar = A[2 * (r * lda + m)], ai = A[2 * (r * lda + m) + 1];
        double br = B[2 * (n * ldb + m)], bi = B[2 * (n * ldb + m) + 1];
        xa_add_prod(&re, ar, br);
        xa_add_prod(&re, -ai, bi);
        xa_add_prod(&im, ar, bi);
        xa_add_prod(&im, ai, br);
      }
      int64_t o = 2 * (r * lds + n);
      xa_round_dd(&re, &hi[o], &lo[o]);
      xa_round_dd(&im, &hi[o + 1], &lo[o + 1]);
    }
  }
}

/* ---- PseudoQuad (double-double) restatement ---------------------------------------------
 * Each helper follows the named routine of PseudoQuad.cuh with __dadd_rn -> +, __dmul_rn -> *,
 * __fma_rn -> fma (no contraction, so the roundings are the same). */
typedef struct {
  double s, t;
} pq;

/* PseudoQuad.cuh:10-15 */
static pq pq_fast2sum(double a, double b) {
  double s = a + b;
  double z = s - a;
  double t = b - z;
  pq r = {s, t};
  return r;
}
/* PseudoQuad.cuh:17-25 */
static pq pq_gen2sum(double a, double b) {
  double s = a + b;
  double ap = s - b;
  double bp = s - ap;
  double da = a - ap;
  double db = b - bp;
  pq r = {s, da + db};
  return r;
}
/* PseudoQuad.cuh:27-31 */
static pq pq_fma2mult(double a, double b) {
  double s = a * b;
  pq r = {s, fma(a, b, -s)};
  return r;
}
/* PseudoQuad.cuh:66-75 ("book" accu) */
static pq pq_accu(pq x, pq y) {
  pq s = pq_gen2sum(x.s, y.s);
  pq t = pq_gen2sum(x.t, y.t);
  double c = s.t + t.s;
  pq v = pq_fast2sum(s.s, c);
  double w = t.t + v.t;
  return pq_fast2sum(v.s, w);
}
/* PseudoQuad.cuh:80-86 */
static pq pq_scale2(pq a, double b) {
  pq p = pq_fma2mult(a.s, b);
  p.t = fma(a.s, 0.0, p.t);
  p.t = fma(a.t, b, p.t);
  return pq_fast2sum(p.s, p.t);
}
/* PseudoQuad.cuh:96-108: compensated multiply-accumulate */
static pq pq_axpy2(pq c, double a, double b) {
  pq r;
  r.s = fma(a, b, c.s);
  double abp = r.s - c.s;
  double cp = r.s - abp;
  double dab = fma(a, b, -abp);
  double dc = c.s - cp;
  r.t = dc + dab;
  r.t = r.t + c.t;
  return r;
}
/* PseudoQuad.cuh:137-140 */
static pq pq_renormalize(pq a) { return pq_fast2sum(a.s, a.t); }
/* PseudoQuad.cuh:149-152 */
static double pq_convert(pq a) { return a.s + a.t; }

void orc_pq_fast2sum(double a, double b, double* s, double* t) { pq r = pq_fast2sum(a, b); *s = r.s; *t = r.t; }
void orc_pq_gen2sum(double a, double b, double* s, double* t) { pq r = pq_gen2sum(a, b); *s = r.s; *t = r.t; }
void orc_pq_fma2mult(double a, double b, double* s, double* t) { pq r = pq_fma2mult(a, b); *s = r.s; *t = r.t; }
void orc_pq_accu(double xs, double xt, double ys, double yt, double* s, double* t) {
  pq x = {xs, xt}, y = {ys, yt};
  pq r = pq_accu(x, y);
  *s = r.s; *t = r.t;
}
void orc_pq_axpy2(double cs, double ct, double a, double b, double* s, double* t) {
  pq c = {cs, ct};
  pq r = pq_axpy2(c, a, b);
  *s = r.s; *t = r.t;
}
void orc_pq_scale2(double as, double at, double b, double* s, double* t) {
  pq a = {as, at};
  pq r = pq_scale2(a, b);
  *s = r.s; *t = r.t;
}

/* Double-double TSMTTSM, in the structure of SPECSMALL<double,PseudoQuad> (specsmall.cuh:28-90)
 * and its deviceReduce (specsmall.cuh:10-26): short axpy2 chains (<= 256 rows, the length one
 * GPU thread covers), chains merged with accu, thread partials merged with accu in thread order,
 * then C = beta*C + convert(scale2(renormalize(sum), alpha)). */
#define PQ_CHAIN 256
void orc_tsmttsm_pq(int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const void* alpha_p,
                    const double* B, int64_t ldb, const void* beta_p, double* C, int64_t ldc,
                    int nthreads) {
  double alpha = *(const double*)alpha_p, beta = *(const double*)beta_p;
  int nt = nthr(nthreads);
  int64_t MN = M * N;
  pq* part = (pq*)calloc((size_t)nt * MN, sizeof(pq));
  pq* chain = (pq*)calloc((size_t)nt * MN, sizeof(pq));
#pragma omp parallel num_threads(nt)
  {
    int t = 0, T = 1;
#ifdef _OPENMP
    t = omp_get_thread_num();
    T = omp_get_num_threads();
#endif
    int64_t k0 = K * t / T, k1 = K * (t + 1) / T;
    pq* p = part + (size_t)t * MN;
    pq* c = chain + (size_t)t * MN;
    for (int64_t kb = k0; kb < k1; kb += PQ_CHAIN) {
      int64_t ke = kb + PQ_CHAIN < k1 ? kb + PQ_CHAIN : k1;
      for (int64_t i = 0; i < MN; i++) c[i].s = c[i].t = 0.0;
      for (int64_t k = kb; k < ke; k++)
        for (int64_t n = 0; n < N; n++)
          for (int64_t m = 0; m < M; m++)
            c[n * M + m] = pq_axpy2(c[n * M + m], A[k * lda + m], B[k * ldb + n]);
      for (int64_t i = 0; i < MN; i++) p[i] = pq_accu(p[i], c[i]);
    }
  }
  for (int64_t n = 0; n < N; n++)
    for (int64_t m = 0; m < M; m++) {
      pq s = {0.0, 0.0};
      for (int t = 0; t < nt; t++) s = pq_accu(s, part[(size_t)t * MN + n * M + m]);
      double v = pq_convert(pq_scale2(pq_renormalize(s), alpha));
      double* out = &C[n * ldc + m];
      *out = (beta == 0.0) ? v : beta * (*out) + v;
    }
  free(part);
  free(chain);
}
