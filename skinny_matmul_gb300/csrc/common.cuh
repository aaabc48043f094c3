// common.cuh -- arithmetic types, accumulation rules and PTX helpers shared by every kernel.
//
// Accumulation rules restate the reference's type-generic helpers:
//   real      acc += a*b                      (cu_complex.h:84-89 axpy)
//   complex   acc += a*b, plain product       (cu_complex.h:127-131, no conjugate)
//   dd        PseudoQuad axpy2 / accu / scale2 / renormalize / convert
//             (PseudoQuad.cuh:96-108, 66-75, 80-86, 137-140, 149-152)
// Epilogue:   C = beta*C + alpha*S, and C = alpha*S (C not read) when beta == 0
//             (genv5.cuh:25, specsmall.cuh:139-140, tsmm/fix3.cuh:31-35).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace skinny {

struct dd {
  double s, t;
};
template <typename R>
struct __align__(2 * sizeof(R)) cplx {
  R x, y;
};
typedef cplx<float> c32;
typedef cplx<double> c64;
// the same storage, marking a TSMTTSM whose left operand is conjugated: C = alpha A^H B + beta C
template <typename R>
struct __align__(2 * sizeof(R)) cplxh {
  R x, y;
};
typedef cplxh<float> c32h;
typedef cplxh<double> c64h;
typedef cplx<dd> zdd;  // double-double real and imaginary parts

// One entry of alpha*B + beta*I (in-place TSMM with M == N: C = A (alpha B + beta I)): alpha*b,
// plus beta on the diagonal (one rounding for real types)
__device__ __forceinline__ float fold_entry(float a, float b, float be, bool diag) {
  return diag ? fmaf(a, b, be) : a * b;
}
__device__ __forceinline__ double fold_entry(double a, double b, double be, bool diag) {
  return diag ? fma(a, b, be) : a * b;
}
template <typename C>
__device__ __forceinline__ C fold_entry_c(C a, C b, C be, bool diag) {
  C r = {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
  if (diag) {
    r.x += be.x;
    r.y += be.y;
  }
  return r;
}
template <typename R>
__device__ __forceinline__ cplx<R> fold_entry(cplx<R> a, cplx<R> b, cplx<R> be, bool diag) {
  return fold_entry_c(a, b, be, diag);
}
template <typename R>
__device__ __forceinline__ cplxh<R> fold_entry(cplxh<R> a, cplxh<R> b, cplxh<R> be, bool diag) {
  return fold_entry_c(a, b, be, diag);
}

// ---------------------------------------------------------------- double-double primitives
__device__ __forceinline__ dd dd_fast2sum(double a, double b) {
  double s = __dadd_rn(a, b);
  double z = __dadd_rn(s, -a);
  return {s, __dadd_rn(b, -z)};
}
__device__ __forceinline__ dd dd_gen2sum(double a, double b) {
  double s = __dadd_rn(a, b);
  double ap = __dadd_rn(s, -b);
  double bp = __dadd_rn(s, -ap);
  double da = __dadd_rn(a, -ap);
  double db = __dadd_rn(b, -bp);
  return {s, __dadd_rn(da, db)};
}
__device__ __forceinline__ dd dd_accu(dd x, dd y) {
  dd s = dd_gen2sum(x.s, y.s);
  dd t = dd_gen2sum(x.t, y.t);
  double c = __dadd_rn(s.t, t.s);
  dd v = dd_fast2sum(s.s, c);
  double w = __dadd_rn(t.t, v.t);
  return dd_fast2sum(v.s, w);
}
__device__ __forceinline__ dd dd_axpy2(dd c, double a, double b) {
  dd r;
  r.s = __fma_rn(a, b, c.s);
  double abp = __dadd_rn(r.s, -c.s);
  double cp = __dadd_rn(r.s, -abp);
  double dab = __fma_rn(a, b, -abp);
  double dc = __dadd_rn(c.s, -cp);
  r.t = __dadd_rn(__dadd_rn(dc, dab), c.t);
  return r;
}
__device__ __forceinline__ dd dd_scale2(dd a, double b) {
  double s = __dmul_rn(a.s, b);
  double t = __fma_rn(a.s, b, -s);
  t = __fma_rn(a.t, b, t);
  return dd_fast2sum(s, t);
}

// ---------------------------------------------------------------- accumulation traits
// Ops<T, Acc>: T is the storage/working type, Acc the accumulator.
template <typename T, typename Acc>
struct Ops;

template <typename R>
struct Ops<R, R> {  // float / double
  static __device__ __forceinline__ R zero() { return R(0); }
  static __device__ __forceinline__ R mac(R acc, R a, R b) { return fma(a, b, acc); }
  static __device__ __forceinline__ R add(R x, R y) { return x + y; }
  static __device__ __forceinline__ bool is_zero(R v) { return v == R(0); }
  static __device__ __forceinline__ R finish(R s, R alpha, R beta, bool beta_zero, const R* c) {
    return beta_zero ? alpha * s : fma(*c, beta, s * alpha);
  }
  // alpha == 1 (decided once per thread by the caller): the same value without the multiply;
  // narrow TSMMs are bound by these epilogue operations on the FP64 pipe
  static __device__ __forceinline__ R finish1(R s, R beta, bool beta_zero, const R* c) {
    return beta_zero ? s : fma(*c, beta, s);
  }
  static __device__ __forceinline__ bool is_one(R a) { return a == R(1); }
  static __device__ __forceinline__ R shfl_xor(R v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
};

template <typename R>
struct Ops<cplx<R>, cplx<R>> {
  typedef cplx<R> C;
  static __device__ __forceinline__ C zero() { return {R(0), R(0)}; }
  static __device__ __forceinline__ C mac(C acc, C a, C b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
    return acc;
  }
  static __device__ __forceinline__ C add(C x, C y) { return {x.x + y.x, x.y + y.y}; }
  static __device__ __forceinline__ C mul(C a, C b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
  // r + beta * c: two FMAs for a real beta (the branch is uniform: beta is a launch argument),
  // which matters where the FP64 pipe bounds the narrow complex TSMM
  static __device__ __forceinline__ C add_beta_c(C r, C beta, C c) {
    if (beta.y == R(0)) return {fma(beta.x, c.x, r.x), fma(beta.x, c.y, r.y)};
    return add(mul(beta, c), r);
  }
  static __device__ __forceinline__ C finish(C s, C alpha, C beta, bool beta_zero, const C* c) {
    C r = mul(alpha, s);
    if (!beta_zero) r = add_beta_c(r, beta, *c);
    return r;
  }
  static __device__ __forceinline__ C finish1(C s, C beta, bool beta_zero, const C* c) {
    return beta_zero ? s : add_beta_c(s, beta, *c);
  }
  static __device__ __forceinline__ bool is_one(C a) { return a.x == R(1) && a.y == R(0); }
  static __device__ __forceinline__ C shfl_xor(C v, int o) {
    return {__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)};
  }
};

template <typename R>
struct Ops<cplxh<R>, cplxh<R>> {  // conj(a) * b per term (A^H B)
  typedef cplxh<R> C;
  static __device__ __forceinline__ C zero() { return {R(0), R(0)}; }
  static __device__ __forceinline__ C mac(C acc, C a, C b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(-a.y, b.x, acc.y);
    return acc;
  }
  static __device__ __forceinline__ C add(C x, C y) { return {x.x + y.x, x.y + y.y}; }
  static __device__ __forceinline__ C mul(C a, C b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
  static __device__ __forceinline__ C finish(C s, C alpha, C beta, bool beta_zero, const C* c) {
    C r = mul(alpha, s);
    if (!beta_zero) r = add(mul(beta, *c), r);
    return r;
  }
  static __device__ __forceinline__ C finish1(C s, C beta, bool beta_zero, const C* c) {
    return beta_zero ? s : add(mul(beta, *c), s);
  }
  static __device__ __forceinline__ bool is_one(C a) { return a.x == R(1) && a.y == R(0); }
  static __device__ __forceinline__ C shfl_xor(C v, int o) {
    return {__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)};
  }
};

template <>
struct Ops<double, dd> {  // double inputs, PseudoQuad accumulation
  static __device__ __forceinline__ dd zero() { return {0.0, 0.0}; }
  static __device__ __forceinline__ dd mac(dd acc, double a, double b) { return dd_axpy2(acc, a, b); }
  static __device__ __forceinline__ dd add(dd x, dd y) { return dd_accu(x, y); }
  static __device__ __forceinline__ double finish(dd s, double alpha, double beta, bool beta_zero,
                                                  const double* c) {
    double v = [&] {
      dd r = dd_fast2sum(s.s, s.t);  // renormalize
      r = dd_scale2(r, alpha);
      return __dadd_rn(r.s, r.t);  // convert
    }();
    return beta_zero ? v : __dadd_rn(__dmul_rn(beta, *c), v);
  }
  static __device__ __forceinline__ double finish1(dd s, double beta, bool beta_zero, const double* c) {
    return finish(s, 1.0, beta, beta_zero, c);
  }
  static __device__ __forceinline__ bool is_one(double) { return false; }
  static __device__ __forceinline__ dd shfl_xor(dd v, int o) {
    return {__shfl_xor_sync(0xffffffffu, v.s, o), __shfl_xor_sync(0xffffffffu, v.t, o)};
  }
};

// The double-double method for the other dtypes (the reference defines PseudoQuad accumulation
// for real FP64 only, types.hpp:49-57): an accumulator in which every product is exact --
// FP64 for FP32 data (a product of two floats fits a double), complex FP64 for complex FP32, and
// PseudoQuad real and imaginary parts for complex FP64 (axpy2 per real product, accu to merge).
// The result is rounded once to the storage type after alpha and beta are applied in the
// accumulator's precision (beta * C in the storage precision's double for complex FP64, as the
// real double-double method does).
template <>
struct Ops<float, double> {
  static __device__ __forceinline__ double zero() { return 0.0; }
  static __device__ __forceinline__ double mac(double acc, float a, float b) {
    return fma((double)a, (double)b, acc);
  }
  static __device__ __forceinline__ double add(double x, double y) { return x + y; }
  static __device__ __forceinline__ float finish(double s, float alpha, float beta, bool beta_zero, const float* c) {
    const double v = (double)alpha * s;
    return (float)(beta_zero ? v : fma((double)*c, (double)beta, v));
  }
  static __device__ __forceinline__ float finish1(double s, float beta, bool beta_zero, const float* c) {
    return (float)(beta_zero ? s : fma((double)*c, (double)beta, s));
  }
  static __device__ __forceinline__ bool is_one(float a) { return a == 1.0f; }
  static __device__ __forceinline__ double shfl_xor(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
};

template <>
struct Ops<c32, c64> {
  static __device__ __forceinline__ c64 zero() { return {0.0, 0.0}; }
  static __device__ __forceinline__ c64 mac(c64 acc, c32 a, c32 b) {
    const double ax = a.x, ay = a.y, bx = b.x, by = b.y;
    acc.x = fma(ax, bx, acc.x);
    acc.x = fma(-ay, by, acc.x);
    acc.y = fma(ax, by, acc.y);
    acc.y = fma(ay, bx, acc.y);
    return acc;
  }
  static __device__ __forceinline__ c64 add(c64 x, c64 y) { return {x.x + y.x, x.y + y.y}; }
  static __device__ __forceinline__ c32 finish(c64 s, c32 alpha, c32 beta, bool beta_zero, const c32* c) {
    const double ar = alpha.x, ai = alpha.y;
    double vr = fma(ar, s.x, -ai * s.y), vi = fma(ar, s.y, ai * s.x);
    if (!beta_zero) {
      const double br = beta.x, bi = beta.y, cr = c->x, ci = c->y;
      vr += fma(br, cr, -bi * ci);
      vi += fma(br, ci, bi * cr);
    }
    return {(float)vr, (float)vi};
  }
  static __device__ __forceinline__ c32 finish1(c64 s, c32 beta, bool beta_zero, const c32* c) {
    return finish(s, {1.0f, 0.0f}, beta, beta_zero, c);
  }
  static __device__ __forceinline__ bool is_one(c32 a) { return a.x == 1.0f && a.y == 0.0f; }
  static __device__ __forceinline__ c64 shfl_xor(c64 v, int o) {
    return {__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)};
  }
};

template <>
struct Ops<c64, zdd> {
  static __device__ __forceinline__ zdd zero() { return {{0.0, 0.0}, {0.0, 0.0}}; }
  static __device__ __forceinline__ zdd mac(zdd acc, c64 a, c64 b) {
    acc.x = dd_axpy2(acc.x, a.x, b.x);
    acc.x = dd_axpy2(acc.x, -a.y, b.y);
    acc.y = dd_axpy2(acc.y, a.x, b.y);
    acc.y = dd_axpy2(acc.y, a.y, b.x);
    return acc;
  }
  static __device__ __forceinline__ zdd add(zdd x, zdd y) { return {dd_accu(x.x, y.x), dd_accu(x.y, y.y)}; }
  static __device__ __forceinline__ c64 finish(zdd s, c64 alpha, c64 beta, bool beta_zero, const c64* c) {
    const dd sr = dd_fast2sum(s.x.s, s.x.t), si = dd_fast2sum(s.y.s, s.y.t);  // renormalize
    const dd re = dd_accu(dd_scale2(sr, alpha.x), dd_scale2(si, -alpha.y));
    const dd im = dd_accu(dd_scale2(sr, alpha.y), dd_scale2(si, alpha.x));
    const double vr = __dadd_rn(re.s, re.t), vi = __dadd_rn(im.s, im.t);  // convert
    if (beta_zero) return {vr, vi};
    return {__dadd_rn(__fma_rn(beta.x, c->x, -beta.y * c->y), vr), __dadd_rn(__fma_rn(beta.x, c->y, beta.y * c->x), vi)};
  }
  static __device__ __forceinline__ c64 finish1(zdd s, c64 beta, bool beta_zero, const c64* c) {
    return finish(s, {1.0, 0.0}, beta, beta_zero, c);
  }
  static __device__ __forceinline__ bool is_one(c64) { return false; }
  static __device__ __forceinline__ zdd shfl_xor(zdd v, int o) {
    return {{__shfl_xor_sync(0xffffffffu, v.x.s, o), __shfl_xor_sync(0xffffffffu, v.x.t, o)},
            {__shfl_xor_sync(0xffffffffu, v.y.s, o), __shfl_xor_sync(0xffffffffu, v.y.t, o)}};
  }
};

// ---------------------------------------------------------------- device error word
// Kernels never trap.  A wait that runs out of iterations records a code here and returns.
enum : int { SKINNY_DEVERR_NONE = 0, SKINNY_DEVERR_TIMEOUT = 1 };

// ---------------------------------------------------------------- PTX helpers (sm_90+ / sm_103a)
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// 1-D bulk copy global -> shared, completion counted on an mbarrier (TMA, no tensor map).
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Default poll limit of a bounded wait.  try_wait itself suspends for a hardware-chosen interval,
// so 2^22 polls is well above a second.
constexpr uint32_t kWaitPolls = 1u << 22;
// Bounded wait: returns false (and records a timeout in *err) after `polls` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int* err,
                                                  uint32_t polls = kWaitPolls) {
  for (uint32_t i = 0; i < polls; i++)
    if (mbar_try_wait(bar, parity)) return true;
  if (err) atomicExch(err, SKINNY_DEVERR_TIMEOUT);
  return false;
}

__host__ __device__ constexpr int ceil_div(int a, int b) { return (a + b - 1) / b; }

}  // namespace skinny
