/* skinny.hpp -- the reference's C++ launcher spellings, forwarding to the C ABI of skinny.h.
 *
 * The reference's call sites name a launcher by namespace and template arguments, e.g.
 *   GENV5::tsmttsm<double, 8, 8>(blockCount, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc)
 *   SPECSMALL::tsmttsm<double, PseudoQuad, 8, 8>(...)
 *   tsmm_fix3<double, 16, 16>(...)
 * (tsmttsm/genv5.cuh:93-96, tsmttsm/specsmall.cuh:94-97, tsmm/fix3.cuh:41-44, listed in
 * versions.hpp:48-177).  This header keeps those spellings as inline functions with the same
 * arguments and return type.  As in the reference, a launcher whose template (M, N) differs from
 * the runtime (varM, varN) returns false without launching; every variant name runs the same
 * kernels here (the variant list is the reference's compile-time tuning space; this library tunes
 * at run time).  T is float, double, cuFloatComplex or cuDoubleComplex; an intermediate type iT
 * other than T with T = double selects double-double accumulation (the reference's PseudoQuad).
 * Launches go to the legacy default stream; blockCount is accepted and ignored.
 *
 * A caller that does not include the reference's PseudoQuad.cuh may write skinny::PseudoQuad. */
#ifndef SKINNY_HPP
#define SKINNY_HPP

#include <cuComplex.h>

#include <cstddef>
#include <type_traits>

#include "skinny.h"

namespace skinny {

struct PseudoQuad {
  double s, t;
};  // tag for double-double accumulation

namespace detail {

inline skinny_c32 c32(cuFloatComplex v) { return skinny_c32{cuCrealf(v), cuCimagf(v)}; }
inline skinny_c64 c64(cuDoubleComplex v) { return skinny_c64{cuCreal(v), cuCimag(v)}; }

template <typename T>
struct abi;

template <>
struct abi<float> {
  static int tsmttsm(size_t bc, int M, int N, int K, const float* A, int lda, float a, const float* B, int ldb,
                     float b, float* C, int ldc) {
    return skinny_tsmttsm_s(bc, M, N, K, A, lda, a, B, ldb, b, C, ldc);
  }
  static int tsmm(size_t bc, int M, int N, int K, const float* A, int lda, float a, const float* B, int ldb,
                  float b, float* C, int ldc) {
    return skinny_tsmm_s(bc, M, N, K, A, lda, a, B, ldb, b, C, ldc);
  }
};

template <>
struct abi<double> {
  static int tsmttsm(size_t bc, int M, int N, int K, const double* A, int lda, double a, const double* B, int ldb,
                     double b, double* C, int ldc) {
    return skinny_tsmttsm_d(bc, M, N, K, A, lda, a, B, ldb, b, C, ldc);
  }
  static int tsmm(size_t bc, int M, int N, int K, const double* A, int lda, double a, const double* B, int ldb,
                  double b, double* C, int ldc) {
    return skinny_tsmm_d(bc, M, N, K, A, lda, a, B, ldb, b, C, ldc);
  }
};

template <>
struct abi<cuFloatComplex> {
  static int tsmttsm(size_t bc, int M, int N, int K, const cuFloatComplex* A, int lda, cuFloatComplex a,
                     const cuFloatComplex* B, int ldb, cuFloatComplex b, cuFloatComplex* C, int ldc) {
    return skinny_tsmttsm_c(bc, M, N, K, reinterpret_cast<const skinny_c32*>(A), lda, c32(a),
                            reinterpret_cast<const skinny_c32*>(B), ldb, c32(b), reinterpret_cast<skinny_c32*>(C), ldc);
  }
  static int tsmm(size_t bc, int M, int N, int K, const cuFloatComplex* A, int lda, cuFloatComplex a,
                  const cuFloatComplex* B, int ldb, cuFloatComplex b, cuFloatComplex* C, int ldc) {
    return skinny_tsmm_c(bc, M, N, K, reinterpret_cast<const skinny_c32*>(A), lda, c32(a),
                         reinterpret_cast<const skinny_c32*>(B), ldb, c32(b), reinterpret_cast<skinny_c32*>(C), ldc);
  }
};

template <>
struct abi<cuDoubleComplex> {
  static int tsmttsm(size_t bc, int M, int N, int K, const cuDoubleComplex* A, int lda, cuDoubleComplex a,
                     const cuDoubleComplex* B, int ldb, cuDoubleComplex b, cuDoubleComplex* C, int ldc) {
    return skinny_tsmttsm_z(bc, M, N, K, reinterpret_cast<const skinny_c64*>(A), lda, c64(a),
                            reinterpret_cast<const skinny_c64*>(B), ldb, c64(b), reinterpret_cast<skinny_c64*>(C), ldc);
  }
  static int tsmm(size_t bc, int M, int N, int K, const cuDoubleComplex* A, int lda, cuDoubleComplex a,
                  const cuDoubleComplex* B, int ldb, cuDoubleComplex b, cuDoubleComplex* C, int ldc) {
    return skinny_tsmm_z(bc, M, N, K, reinterpret_cast<const skinny_c64*>(A), lda, c64(a),
                         reinterpret_cast<const skinny_c64*>(B), ldb, c64(b), reinterpret_cast<skinny_c64*>(C), ldc);
  }
};

template <typename T, typename iT>
inline bool tsmttsm(size_t bc, int M, int N, int K, const T* A, int lda, T a, const T* B, int ldb, T b, T* C,
                    int ldc) {
  if constexpr (std::is_same<T, double>::value && !std::is_same<iT, double>::value)
    return skinny_tsmttsm_dd(bc, M, N, K, A, lda, a, B, ldb, b, C, ldc) != 0;
  else
    return abi<T>::tsmttsm(bc, M, N, K, A, lda, a, B, ldb, b, C, ldc) != 0;
}

template <typename T>
inline bool tsmm(size_t bc, int M, int N, int K, const T* A, int lda, T a, const T* B, int ldb, T b, T* C, int ldc) {
  return abi<T>::tsmm(bc, M, N, K, A, lda, a, B, ldb, b, C, ldc) != 0;
}

}  // namespace detail
}  // namespace skinny

/* TSMTTSM variants: namespace::tsmttsm<T, [iT,] M, N[, extra]>(blockCount, varM, varN, K, ...) */
#define SKINNY_TSMTTSM_T_MN(NS)                                                                      \
  namespace NS {                                                                                     \
  template <typename T, int M, int N>                                                                \
  inline bool tsmttsm(const size_t blockCount, const int varM, const int varN, const int K,          \
                      const T* A, const int lda, const T alpha, const T* B, const int ldb,           \
                      const T beta, T* C, const int ldc) {                                           \
    if (varM != M || varN != N) return false;                                                        \
    return skinny::detail::tsmttsm<T, T>(blockCount, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc);  \
  }                                                                                                  \
  }
#define SKINNY_TSMTTSM_T_IT_MN(NS)                                                                   \
  namespace NS {                                                                                     \
  template <typename T, typename iT, int M, int N>                                                   \
  inline bool tsmttsm(const size_t blockCount, const int varM, const int varN, const int K,          \
                      const T* A, const int lda, const T alpha, const T* B, const int ldb,           \
                      const T beta, T* C, const int ldc) {                                           \
    if (varM != M || varN != N) return false;                                                        \
    return skinny::detail::tsmttsm<T, iT>(blockCount, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc); \
  }                                                                                                  \
  }

SKINNY_TSMTTSM_T_MN(GENV5)
SKINNY_TSMTTSM_T_MN(GENV6)
SKINNY_TSMTTSM_T_MN(GENV32)
SKINNY_TSMTTSM_T_IT_MN(GENV7)
SKINNY_TSMTTSM_T_IT_MN(SPECSMALL)
SKINNY_TSMTTSM_T_IT_MN(REDUCEONLY)

namespace GENV1 {
enum class MEMPATH { GLOBAL, TEX };
template <typename T, int M, int N, MEMPATH P>
inline bool tsmttsm(const size_t bc, const int varM, const int varN, const int K, const T* A, const int lda,
                    const T alpha, const T* B, const int ldb, const T beta, T* C, const int ldc) {
  if (varM != M || varN != N) return false;
  return skinny::detail::tsmttsm<T, T>(bc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc);
}
}  // namespace GENV1
namespace GENV4 {
enum class MEMPATH { GLOBAL, TEX };
template <typename T, int M, int N, MEMPATH P>
inline bool tsmttsm(const size_t bc, const int varM, const int varN, const int K, const T* A, const int lda,
                    const T alpha, const T* B, const int ldb, const T beta, T* C, const int ldc) {
  if (varM != M || varN != N) return false;
  return skinny::detail::tsmttsm<T, T>(bc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc);
}
}  // namespace GENV4
namespace GENV3 {
enum class MEMPATH { GLOBAL, TEX };
template <typename T, typename iT, int M, int N, MEMPATH P>
inline bool tsmttsm(const size_t bc, const int varM, const int varN, const int K, const T* A, const int lda,
                    const T alpha, const T* B, const int ldb, const T beta, T* C, const int ldc) {
  if (varM != M || varN != N) return false;
  return skinny::detail::tsmttsm<T, iT>(bc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc);
}
}  // namespace GENV3
namespace GENV3X {
template <typename T, int M, int N, int THREAD_PER_N>
inline bool tsmttsm(const size_t bc, const int varM, const int varN, const int K, const T* A, const int lda,
                    const T alpha, const T* B, const int ldb, const T beta, T* C, const int ldc) {
  if (varM != M || varN != N) return false;
  return skinny::detail::tsmttsm<T, T>(bc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc);
}
}  // namespace GENV3X
namespace GENV8 {
template <typename T, typename iT, int M, int N, int tileSize>
inline bool tsmttsm(const size_t bc, const int varM, const int varN, const int K, const T* A, const int lda,
                    const T alpha, const T* B, const int ldb, const T beta, T* C, const int ldc) {
  if (varM != M || varN != N) return false;
  return skinny::detail::tsmttsm<T, iT>(bc, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc);
}
}  // namespace GENV8

/* TSMM variants: fixed (M, N) template forms and the variable-size forms */
#define SKINNY_TSMM_FIX(NAME)                                                                           \
  template <typename T, int M, int N>                                                                   \
  inline bool NAME(const size_t blockCount, const int varM, const int varN, const int K, const T* A,    \
                   const int lda, const T alpha, const T* B, const int ldb, const T beta, T* C,         \
                   const int ldc) {                                                                     \
    if (varM != M || varN != N) return false;                                                           \
    return skinny::detail::tsmm<T>(blockCount, M, N, K, A, lda, alpha, B, ldb, beta, C, ldc);           \
  }
#define SKINNY_TSMM_VAR(NAME)                                                                           \
  template <typename T>                                                                                 \
  inline bool NAME(const size_t blockCount, const int varM, const int varN, const int K, const T* A,    \
                   const int lda, const T alpha, const T* B, const int ldb, const T beta, T* C,         \
                   const int ldc) {                                                                     \
    return skinny::detail::tsmm<T>(blockCount, varM, varN, K, A, lda, alpha, B, ldb, beta, C, ldc);     \
  }

SKINNY_TSMM_FIX(tsmm_fix1)
SKINNY_TSMM_FIX(tsmm_fix2)
SKINNY_TSMM_FIX(tsmm_fix3)
SKINNY_TSMM_FIX(tsmm_fix4)
SKINNY_TSMM_FIX(tsmm_fix_fb)
SKINNY_TSMM_FIX(tsmm_fix_blend)
SKINNY_TSMM_FIX(tsmm_fix_ip_ghost)
SKINNY_TSMM_VAR(tsmm_var1)
SKINNY_TSMM_VAR(tsmm_var_ip_ghost)
SKINNY_TSMM_VAR(tsmm_varip1)
SKINNY_TSMM_VAR(tsmm_varip2)
SKINNY_TSMM_VAR(tsmm_varip3)
SKINNY_TSMM_VAR(tsmm_varip_blend)

#undef SKINNY_TSMTTSM_T_MN
#undef SKINNY_TSMTTSM_T_IT_MN
#undef SKINNY_TSMM_FIX
#undef SKINNY_TSMM_VAR

#endif /* SKINNY_HPP */
