/* Device-only translation unit that compiles the REFERENCE's own kernels for sm_103a.
 *
 * Test infrastructure, not product code: oracle/Makefile (target `ref`) compiles this file with
 * the reference tree on the include path into oracle/_ref/ref_kernels_<part>.cubin, and
 * oracle/ref_runner.cpp loads those cubins on the GPU and launches the kernels with the launch
 * configuration of the reference's own launchers.  Nothing here restates a kernel: every kernel
 * is the reference's header, unmodified; this file only names which template instantiations to
 * emit (host code referencing a __global__ template makes nvcc compile that instantiation).
 *
 * Instantiated (reference file:lines of the launcher whose kernel choice is mirrored):
 *   TSMTTSM  GENV5     tsmttsm/genv5.cuh:93-114     blockProductKernel<T,M,N,256,false> or, for
 *                                                   N > M, <T,N,M,256,true>; deviceReduce<T,M,N>
 *            GENV3X    tsmttsm/genv3x.cuh:83-106    the same with THREAD_PER_N = 2 ("FGEN32T",
 *                                                   versions.hpp:129-131)
 *            SPECSMALL tsmttsm/specsmall.cuh:94-125 <T,iT,M,N,256,false,SELF> or, for N > M,
 *                                                   <T,iT,N,M,256,true,false>; deviceReduce<T,iT,M,N>
 *                                                   (specsmall.cuh:10-26), iT = double, PseudoQuad
 *   TSMM     FIX3      tsmm/fix3.cuh:41-65          tsmm_fix3_kernel<T,M,N,BS,BETAISZERO>,
 *                                                   BS = M*N*8 > 10240 ? 256 : 128
 *            FIX_FB    tsmm/fix_fb.cuh:72-102       tsmm_fix_fb_kernel<T,M,N,BS,BETAISZERO>,
 *                                                   BS = M*N > 1024 ? 1024 : 256
 *            FIX_IP_GHOST tsmm/fix_ip_ghost.cuh:24-44 fix_ip_ghost_kernel<T,N,M>
 * Not built: GENV6 (tsmttsm/genv6.cuh:67-89).  Its kernel reads BCache[i * N + n]
 * (genv6.cuh:54) with n up to rowsPerBlock - 1, past the N * rowsPerBlock entries of that shared
 * array, whenever K >= rowsPerBlock; on GB300 that out-of-range shared-memory read faulted
 * (illegal memory access), so it is never launched.
 * Types: double (all), float (GENV5, SPECSMALL<float,float>, FIX3), cuDoubleComplex
 * (FIX_IP_GHOST, which is complex-clean; FIX3 / GENV5 / SPECSMALL are real-only).
 *
 * REF_PART selects a slice of the list so the parts compile in parallel.
 */
#include <cuda_runtime.h>
#include <cuComplex.h>

#include <vector>

// The GENV launchers size their static workspace with the harness's global `dtype`
// (types.hpp:52-55); it must exist for their host code to parse.
typedef double dtype;

#include "tsmttsm/genv5.cuh"
#include "tsmttsm/genv3x.cuh"
#include "tsmttsm/specsmall.cuh"
#include "tsmm/fix3.cuh"
#include "tsmm/fix_fb.cuh"
#include "tsmm/fix_ip_ghost.cuh"

#ifndef REF_PART
#define REF_PART 0
#endif

namespace {

using Uses = std::vector<const void*>;

template <typename T, int M, int N>
void genv5(Uses& v) {
  if constexpr (N > M)
    v.push_back((const void*)GENV5::blockProductKernel<T, N, M, 256, true>);
  else
    v.push_back((const void*)GENV5::blockProductKernel<T, M, N, 256, false>);
  v.push_back((const void*)GENV5::deviceReduce<T, M, N>);
}

template <typename T, int M, int N>
void genv3x(Uses& v) {
  if constexpr (N > M)
    v.push_back((const void*)GENV3X::blockProductKernel<T, N, M, 256, true, 2>);
  else
    v.push_back((const void*)GENV3X::blockProductKernel<T, M, N, 256, false, 2>);
  v.push_back((const void*)GENV3X::deviceReduce<T, M, N>);
}

template <typename T, typename iT, int M, int N>
void specsmall(Uses& v) {
  if constexpr (N > M) {
    v.push_back((const void*)SPECSMALL::blockProductKernel<T, iT, N, M, 256, true, false>);
  } else {
    v.push_back((const void*)SPECSMALL::blockProductKernel<T, iT, M, N, 256, false, false>);
    if constexpr (M == N)
      v.push_back((const void*)SPECSMALL::blockProductKernel<T, iT, M, N, 256, false, true>);
  }
  v.push_back((const void*)SPECSMALL::deviceReduce<T, iT, M, N>);
}

template <typename T, int M, int N>
void fix3(Uses& v) {
  constexpr int BS = (M * N * 8 > 10 * 1024) ? 256 : 128;
  v.push_back((const void*)tsmm_fix3_kernel<T, M, N, BS, true>);
  v.push_back((const void*)tsmm_fix3_kernel<T, M, N, BS, false>);
}

template <typename T, int M, int N>
void fix_fb(Uses& v) {
  constexpr int BS = (M * N > 1024) ? 1024 : 256;
  v.push_back((const void*)tsmm_fix_fb_kernel<T, M, N, BS, true>);
  v.push_back((const void*)tsmm_fix_fb_kernel<T, M, N, BS, false>);
}

template <typename T, int M, int N>
void fix_ip_ghost(Uses& v) {
  v.push_back((const void*)fix_ip_ghost_kernel<T, N, M>);
}

// TSMTTSM shapes: the golden integer fixtures' widths plus C1 (8 x 8); all <= 32 (GENV5 and
// SPECSMALL refuse wider, genv5.cuh:99, specsmall.cuh:99).
#define TS_SHAPES(X, ...)                                                                        \
  X(__VA_ARGS__, 1, 1) X(__VA_ARGS__, 2, 2) X(__VA_ARGS__, 3, 3) X(__VA_ARGS__, 4, 4)              \
  X(__VA_ARGS__, 8, 8) X(__VA_ARGS__, 5, 7) X(__VA_ARGS__, 4, 16) X(__VA_ARGS__, 16, 4)            \
  X(__VA_ARGS__, 8, 32) X(__VA_ARGS__, 16, 16) X(__VA_ARGS__, 32, 32) X(__VA_ARGS__, 1, 8)         \
  X(__VA_ARGS__, 13, 3)
// TSMM shapes: the same plus the C2 widths 64 x 64.
#define TSMM_SHAPES(X, ...) TS_SHAPES(X, __VA_ARGS__) X(__VA_ARGS__, 64, 64)

#define USE_MN(fn, T, M, N) fn<T, M, N>(v);
#define USE_IT_MN(fn, T, IT, M, N) fn<T, IT, M, N>(v);

}  // namespace

// Referenced nowhere; its body is what makes nvcc emit the instantiations above.
void ref_kernel_instantiations() {
  Uses v;
#if REF_PART == 0
  TS_SHAPES(USE_MN, genv5, double)
  TS_SHAPES(USE_MN, genv3x, double)
  TS_SHAPES(USE_MN, genv5, float)
#elif REF_PART == 1
  TS_SHAPES(USE_IT_MN, specsmall, double, double)
  TS_SHAPES(USE_IT_MN, specsmall, float, float)
#elif REF_PART == 2
  TS_SHAPES(USE_IT_MN, specsmall, double, PseudoQuad)
#elif REF_PART == 3
  TSMM_SHAPES(USE_MN, fix3, double)
  TSMM_SHAPES(USE_MN, fix3, float)
#elif REF_PART == 4
  TSMM_SHAPES(USE_MN, fix_fb, double)
  TSMM_SHAPES(USE_MN, fix_ip_ghost, double)
  TSMM_SHAPES(USE_MN, fix_ip_ghost, cuDoubleComplex)
#endif
  (void)v;
}
