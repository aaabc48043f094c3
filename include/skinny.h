/* skinny.h -- C ABI of the GB300 (sm_103a) tall-skinny product library.
 *
 * Drop-in boundary for te42kyfo/skinny_matmul's templated launchers, whose common shape is
 * MatmulFunctionType (versions.hpp:43-45):
 *   bool f(size_t blockCount, int M, int N, int K, const T* A, int lda, T alpha,
 *          const T* B, int ldb, T beta, T* C, int ldc)
 *
 * Layouts (unchanged from the reference; all pointers are DEVICE pointers owned by the caller):
 *   TSMTTSM  C[n*ldc+m] = alpha * sum_k A[k*lda+m] * B[k*ldb+n] + beta * C[n*ldc+m]
 *            A: K x M row-major, B: K x N row-major, C: M x N with column stride ldc.
 *            A == B with lda == ldb and M == N is the Gram (SELF) mode.
 *   TSMM     C[r*ldc+n] = alpha * sum_m A[r*lda+m] * B[n*ldb+m] + beta * C[r*ldc+n]
 *            A: K x M row-major, B: M x N stored column by column (B[n*ldb+m]), C: K x N.
 *            A == C (with lda == ldc) is the in-place form; each output row is computed from
 *            that row's old contents.
 *   Complex values are interleaved (re, im) as cuFloatComplex / cuDoubleComplex; products use
 *   the plain transpose, not the conjugate (the reference's cuBLAS oracle uses OP_T,
 *   tsmttsm/gen_cublas.cuh:29-39).
 *   beta == 0 means C is not read (tsmm/fix3.cuh:31-35 BETAISZERO; BLAS convention).
 *
 * Differences from the reference, all deliberate:
 *   - every call returns a status and never exits the process (the reference aborts through
 *     GPU_ERROR, gpu_error.cuh:4-13);
 *   - sizes and leading dimensions are 64-bit in the skinny_* entry points;
 *   - M and N are runtime values (the reference compiles one binary per (M, N), Makefile:11-20);
 *   - calls are stream-ordered on the stream given; the reference-shaped entry points use the
 *     legacy default stream, as the reference does;
 *   - workspace is owned by a handle, one buffer per stream, so concurrent streams never share a
 *     partial-sum buffer (the reference keeps one static buffer per kernel family,
 *     tsmttsm/genv5.cuh:91).
 */
#ifndef SKINNY_H
#define SKINNY_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  SKINNY_OK = 0,
  SKINNY_UNSUPPORTED = 1, /* shape / dtype / method combination not provided (reference: return false) */
  SKINNY_BAD_ARG = 2,     /* invalid sizes, leading dimensions, null pointers or aliasing */
  SKINNY_NO_MEM = 3,      /* workspace allocation failed or request over the memory budget */
  SKINNY_TIMEOUT = 4,     /* a bounded device-side wait gave up; the device stays usable */
  SKINNY_DEVICE_ERROR = 5,/* CUDA reported an error */
  SKINNY_NOT_READY = 6    /* request-loop ticket not finished yet */
} skinny_status;

typedef enum {
  SKINNY_R32 = 0, /* float                       */
  SKINNY_R64 = 1, /* double                      */
  SKINNY_C32 = 2, /* cuFloatComplex  (float re, im)  */
  SKINNY_C64 = 3  /* cuDoubleComplex (double re, im) */
} skinny_dtype;

typedef enum {
  SKINNY_ACC_NATIVE = 0, /* accumulate in the working type (reference dItype == dtype) */
  SKINNY_ACC_DD = 1,     /* exact-product accumulation: R64 double-double (reference dItype == PseudoQuad,
                            types.hpp:49-57), C64 double-double real and imaginary parts, R32 / C32 in
                            FP64 / complex FP64; not for the conjugate product */
  SKINNY_ACC_SPLIT = 2,  /* split precision: values sliced into FP16 digits, products on tcgen05
                            tensor cores with exact FP32 accumulation, recombined in FP64.  R64, C64,
                            and R32 / C32 storage (widened exactly, rounded once to FP32) at the same
                            widths.  No counterpart in the reference. */
  SKINNY_ACC_AUTO = 3    /* fastest method meeting the working precision's error bound */
} skinny_acc;

typedef struct { float x, y; } skinny_c32;  /* same layout as cuFloatComplex  */
typedef struct { double x, y; } skinny_c64; /* same layout as cuDoubleComplex */

typedef struct skinny_handle_st* skinny_handle;

/* Handle: device, per-stream workspaces, autotune table.  One handle may be used from several
 * host threads; calls on the same stream are serialised in stream order. */
skinny_status skinny_create(skinny_handle* handle, int device);
skinny_status skinny_destroy(skinny_handle handle);
const char* skinny_status_string(skinny_status s);
/* Detail message of the last failing call on this host thread ("" if none). */
const char* skinny_last_error(void);
/* Synchronises the device and reports SKINNY_TIMEOUT if a kernel's bounded wait gave up since
 * the last check (the flag is then cleared and the handle's workspaces are reset). */
skinny_status skinny_check_device(skinny_handle handle);
/* Poll limit of the CUDA-core TSMTTSM kernel's bounded waits on its copy ring (default
 * 4194304 polls, each suspending for a hardware-chosen interval: well above a second).  A wait
 * that runs out records a timeout for skinny_check_device; its CTA first waits, with the default
 * bound, for the copies it has already issued, then exits without writing C.  0 makes every such
 * wait give up at once, which exercises that path without a fault.  No counterpart in the
 * reference (its kernels have no waits that can time out). */
skinny_status skinny_set_wait_limit(skinny_handle handle, uint32_t polls);

/* Number of kernels this library has launched in this process (all devices, all handles);
 * lets a caller count device launches inside a timed region.  No counterpart in the reference. */
uint64_t skinny_kernel_launches(void);

/* TSMTTSM, replaces tsmttsm/genv{3,3x,5,6,7,8}.cuh, specsmall.cuh (+ their deviceReduce) and
 * tsmttsm/gen_cublas.cuh:12-46.  alpha/beta point to one HOST value of the dtype. */
skinny_status skinny_tsmttsm(skinny_handle handle, skinny_dtype dtype, skinny_acc acc, int64_t M,
                             int64_t N, int64_t K, const void* A, int64_t lda, const void* alpha,
                             const void* B, int64_t ldb, const void* beta, void* C, int64_t ldc,
                             void* stream);

/* TSMM, replaces tsmm/fix{1,2,3,4}.cuh, fix_fb.cuh, var1.cuh, varip{1,2,3}.cuh,
 * fix_ip_ghost.cuh, var_ip_ghost.cuh, the blends (fix_blend.cuh:7-29, varip_blend.cuh:8-29) and
 * tsmm/cublas.cuh:18-62. */
skinny_status skinny_tsmm(skinny_handle handle, skinny_dtype dtype, skinny_acc acc, int64_t M,
                          int64_t N, int64_t K, const void* A, int64_t lda, const void* alpha,
                          const void* B, int64_t ldb, const void* beta, void* C, int64_t ldc,
                          void* stream);
/* C = alpha A^H B + beta C: the conjugate transpose of A (Hermitian Gram when A == B).  No
 * counterpart in the reference, whose complex TSMTTSM uses the plain transpose (cuBLAS OP_T,
 * tsmttsm/gen_cublas.cuh:29-39); complex orthogonalisation needs this form.  Same arguments as
 * skinny_tsmttsm; for real dtypes identical to it.  Methods: native, auto, split (complex FP64,
 * M, N <= 64). */
skinny_status skinny_tsmttsm_conj(skinny_handle handle, skinny_dtype dtype, skinny_acc acc, int64_t M, int64_t N,
                                  int64_t K, const void* A, int64_t lda, const void* alpha, const void* B, int64_t ldb,
                                  const void* beta, void* C, int64_t ldc, void* stream);

/* SVQB orthogonalisation of X (K x M row-major, ldx >= M, FP64), in place, entirely on the
 * device; replaces svqb/svqb.cu:72-130 (which runs the eigensolve on the host through MAGMA).
 *   S = X^T X (gram_acc selects the method), d_i = 1/sqrt(S_ii) (0 if S_ii <= 1e-15),
 *   S <- D S D, S = U L U^T (Jacobi, FP64), T = D U diag(1/sqrt(max(1e-15, l))),
 *   X <- X T (in-place TSMM).
 * If orth_err_out is non-null, ||Q^T Q - I||_F is computed on the device (double-double Gram)
 * and written there after a stream synchronisation (svqb/svqb.cu:184-211 getL2Error). */
skinny_status skinny_svqb(skinny_handle handle, skinny_acc gram_acc, int64_t K, int64_t M,
                          double* X, int64_t ldx, double* orth_err_out, void* stream);

/* SVQB in double-double on the host: the reference's high-precision study (svqb/svqb.cu:132-182,
 * svqb_xd<dd_real> through MPACK's Rgemm / Rsyev), an accuracy baseline for skinny_svqb.
 * X (input) and Q (output) are HOST arrays, K x M row-major (ld = M), M <= 256; the Gram
 * S = X^T X, the scaling D^-1/2 (0 where S_ii <= 2^-104), the eigensolve (cyclic Jacobi in place of
 * Rsyev; ascending eigenvalues, each vector's largest entry positive), T = D U Lambda^-1/2 and
 * Q = X T all run in double-double arithmetic on `threads` host threads (<= 0: all hardware
 * threads); Q is rounded to double once.  Touches no GPU.  orth_err_out (nullable):
 * ||Q^T Q - I||_F of the rounded Q with a double-double Gram. */
skinny_status skinny_svqb_host_dd(const double* X, double* Q, int64_t K, int M, int threads, double* orth_err_out);

/* CholQR (passes = 1) / CholQR2 (passes = 2) of X (K x M, FP64, M <= 64) in place: per pass the
 * Gram S = X^T X (method gram_acc), the Cholesky S = R^T R and X <- X R^-1 by the in-place TSMM,
 * all on the device.  No counterpart in the reference (its orthogonalisation is SVQB); the same
 * building blocks.  SKINNY_BAD_ARG when a Gram is not numerically positive definite.
 * orth_err_out (nullable): ||Q^T Q - I||_F with a double-double Gram (synchronises the stream). */
skinny_status skinny_cholqr(skinny_handle handle, skinny_acc gram_acc, int64_t K, int64_t M, double* X, int64_t ldx,
                            int passes, double* orth_err_out, void* stream);

/* SVQB of a complex FP64 block X (K x M, interleaved, M <= 64) in place: Hermitian Gram
 * S = X^H X (skinny_tsmttsm_conj, method gram_acc), Hermitian Jacobi eigensolve on the device,
 * X <- X (D^-1/2 U Lambda^-1/2) by the complex in-place TSMM.  No counterpart in the reference
 * (its SVQB is real).  orth_err_out (nullable): ||Q^H Q - I||_F (synchronises the stream). */
skinny_status skinny_svqb_z(skinny_handle handle, skinny_acc gram_acc, int64_t K, int64_t M, void* X, int64_t ldx,
                            double* orth_err_out, void* stream);

/* FP64 TSMTTSM that allocates nothing.  No counterpart in the reference.
 * For callers that cannot call cudaMalloc: code that runs under an allocator owning the whole
 * device pool, or a latency-critical path where cudaMalloc's implicit device synchronisation is
 * not allowed, cannot create a skinny_handle (whose workspaces are cudaMalloc'ed).  This entry
 * point runs the FP64 TSMTTSM kernel with its scratch in a fixed 16 MiB device array inside the
 * library (held by every GPU that loads the library until the process exits); A, B and C are
 * still the caller's.  It uses the current device and the given stream.
 *   - The first call on a device looks up the array's device address; make it before any stream
 *     capture.
 *   - M*N <= 1048576 (2^20, the most the CUDA-core kernel's reduction handles in FP64), else
 *     SKINNY_BAD_ARG before any device work; within that, shapes whose row tile does not fit in
 *     shared memory (M + N above about 1800 when A != B) return SKINNY_UNSUPPORTED, as in
 *     skinny_tsmttsm.  For large M*N the grid is reduced so the partials fit in the array.
 *   - Every call shares the one array (its ticket counters are cleared on the stream at each
 *     call): calls that overlap on the GPU race and must be ordered by the caller.
 *   - A bounded device-side wait that times out leaves C unwritten; it is reported by
 *     skinny_tsmttsm_d_static_check, not by this call (which returns before the kernel runs). */
skinny_status skinny_tsmttsm_d_static(int64_t M, int64_t N, int64_t K, const double* A,
                                      int64_t lda, double alpha, const double* B, int64_t ldb,
                                      double beta, double* C, int64_t ldc, void* stream);
/* Status of the skinny_tsmttsm_d_static calls on the current device: synchronises `stream`, then
 * returns SKINNY_TIMEOUT (and clears the flag) if a bounded wait of any call since the last check
 * timed out, else SKINNY_OK.  Allocates nothing. */
skinny_status skinny_tsmttsm_d_static_check(void* stream);

/* Autotuner.  Replaces the reference's compile-time choice of one kernel variant per (M, N)
 * (versions.hpp:48-177, multi_dispatch.cuh, tsmm/fix_blend.cuh:7-29): for (op, dtype, acc, M, N)
 * it times the candidate launch shapes (CTAs per SM, rows per tile) and, for SKINNY_ACC_AUTO on
 * R64, the split-precision against the CUDA-core method, on scratch operands of K rows, and
 * records the fastest in the handle's table; later calls with that key use it.
 * op: 0 = TSMTTSM, 1 = TSMM.  Synchronises `stream`; allocates and frees its scratch. */
skinny_status skinny_autotune(skinny_handle handle, int op, skinny_dtype dtype, skinny_acc acc,
                              int64_t M, int64_t N, int64_t K, void* stream);
/* The tuned table as JSON text (buf of len bytes; *written = bytes needed incl. the NUL). */
skinny_status skinny_tune_export(skinny_handle handle, char* buf, size_t len, size_t* written);
/* Merge a table produced by skinny_tune_export. */
skinny_status skinny_tune_import(skinny_handle handle, const char* json);

/* ---- Request loop (continuous batching).  No counterpart in the reference.
 * A server accepts TSMTTSM / TSMM / SVQB requests on HOST buffers as they arrive, admits them in
 * arrival order while their device bytes fit the memory budget and an in-flight slot is free,
 * runs each (upload, product, download) on one of its streams so that the work of requests in
 * flight overlaps on the device, and retires them as their completion events fire; admission
 * continues while others run.  Host buffers must stay valid until the ticket completes; pinned
 * host memory lets uploads and downloads overlap with compute.  Requests flagged `device` name
 * operands already resident in HBM: the server then only schedules them (admission counts their
 * operand bytes against the budget) and runs the product on them in place.  A server created with a NULL
 * handle runs in dry mode: nothing touches a device and each request "runs" for a time
 * proportional to its bytes (for testing the scheduling logic without a GPU). */
typedef enum { SKINNY_OP_TSMTTSM = 0, SKINNY_OP_TSMM = 1, SKINNY_OP_SVQB = 2 } skinny_op;

typedef struct {
  skinny_op op;
  skinny_dtype dtype;
  skinny_acc acc;
  int64_t M, N, K;
  const void* A; /* host; SVQB: X (K x M), updated in place through C */
  int64_t lda;
  const void* B; /* host; unused for SVQB */
  int64_t ldb;
  void* C;       /* host; read when beta != 0, always written; SVQB: X */
  int64_t ldc;
  double alpha[2], beta[2]; /* (re, im); real dtypes use [0] */
  int32_t device; /* 0: A, B, C are host buffers (uploaded and downloaded by the server);
                     1: device buffers resident in HBM, used in place (nothing copied) */
} skinny_request;

typedef struct {
  uint64_t submitted, completed, failed, rejected;
  double p50_latency_us, p99_latency_us, mean_latency_us;
  double bytes; /* algorithmic bytes of the completed requests */
  double busy_seconds; /* wall time from the first admission to the last completion */
  uint64_t peak_bytes_in_use;
  uint64_t max_inflight_seen;
  uint64_t grouped;        /* requests that ran in grouped launches */
  uint64_t group_launches; /* grouped launches (graph replays) */
} skinny_server_stats;

typedef struct skinny_server_st* skinny_server;

skinny_status skinny_server_create(skinny_server* server, skinny_handle handle, uint64_t mem_budget_bytes,
                                   int num_streams, int max_inflight);
/* Queue a request; *ticket identifies it.  SKINNY_NO_MEM if it can never fit the budget. */
skinny_status skinny_server_submit(skinny_server server, const skinny_request* request, uint64_t* ticket);
/* SKINNY_NOT_READY while the ticket runs; otherwise SKINNY_OK with *result = the request's status. */
skinny_status skinny_server_poll(skinny_server server, uint64_t ticket, skinny_status* result);
/* Block until the ticket completes or timeout_s passes (SKINNY_TIMEOUT). */
skinny_status skinny_server_wait(skinny_server server, uint64_t ticket, skinny_status* result,
                                 double timeout_s);
skinny_status skinny_server_drain(skinny_server server, double timeout_s);
skinny_status skinny_server_stats_get(skinny_server server, skinny_server_stats* stats);
skinny_status skinny_server_destroy(skinny_server server); /* drains first */
/* Small requests -- TSMTTSM / TSMM with the native or auto method, M, N <= 64 and a cost of at
 * most max_request_bytes, the cost being the larger of the request's algorithmic bytes and its
 * FMAs priced at the dtype's HBM-to-FMA rate ratio (about 11 bytes per FP64 FMA on GB300) --
 * do not take an in-flight slot: as they are admitted they
 * are packed into grouped launches (skinny_group) of up to max_group requests, one launch per
 * dtype present, replayed from instantiated CUDA graphs on a high-priority stream (the graph's
 * descriptor copy and kernel nodes are updated and switched on or off per batch; two graphs
 * alternate so that a batch is prepared while the previous one runs).  Small requests may pass a
 * large one that waits for a slot, never one that waits for memory.  Default 32 MiB and 512;
 * max_request_bytes = 0 turns grouping off (every request then runs as its own launch). */
skinny_status skinny_server_set_grouping(skinny_server server, uint64_t max_request_bytes, int32_t max_group);

/* ---- Grouped launches.  No counterpart in the reference.
 * One persistent launch runs `count` small products of one dtype.  Each item is a TSMTTSM or a
 * TSMM with the layouts and argument meaning of skinny_tsmttsm / skinny_tsmm (device pointers,
 * in-place TSMM and Gram TSMTTSM included), M, N <= 64, any K; alpha and beta are (re, im)
 * doubles, rounded to float for the FP32 dtypes.  Items' rows are cut into units spread over the
 * grid; a TSMTTSM sums its units' partials in unit order inside the launch, so every result is
 * deterministic and does not depend on the other items.  CUDA-core arithmetic in the working
 * precision (the native method); a TSMM item gives the same bits as skinny_tsmm with the native
 * method.  Items must not write memory that another item of the batch reads. */
typedef struct {
  skinny_op op; /* SKINNY_OP_TSMTTSM or SKINNY_OP_TSMM */
  int64_t M, N, K;
  const void* A;
  int64_t lda;
  const void* B;
  int64_t ldb;
  void* C;
  int64_t ldc;
  double alpha[2], beta[2];
} skinny_group_item;

skinny_status skinny_group(skinny_handle handle, skinny_dtype dtype, const skinny_group_item* items, int32_t count,
                           void* stream);

/* ---- Reference-shaped entry points ---------------------------------------------------------
 * Exactly MatmulFunctionType (versions.hpp:43-45).  They run on the legacy default stream with a
 * per-device default handle, like the reference's launchers (e.g. tsmttsm/genv5.cuh:93-114,
 * tsmm/fix3.cuh:41-65).  Return 1 when the product was launched, 0 when it was not (unsupported
 * shape, or an error: see skinny_last_error()).  blockCount is accepted for signature
 * compatibility and ignored: the grid is sized from the SM count.
 * The _dd variants take double data and accumulate in double-double (the reference's
 * dItype == PseudoQuad). */
int skinny_tsmttsm_s(size_t blockCount, int M, int N, int K, const float* A, int lda, float alpha,
                     const float* B, int ldb, float beta, float* C, int ldc);
int skinny_tsmttsm_d(size_t blockCount, int M, int N, int K, const double* A, int lda, double alpha,
                     const double* B, int ldb, double beta, double* C, int ldc);
int skinny_tsmttsm_c(size_t blockCount, int M, int N, int K, const skinny_c32* A, int lda,
                     skinny_c32 alpha, const skinny_c32* B, int ldb, skinny_c32 beta, skinny_c32* C,
                     int ldc);
int skinny_tsmttsm_z(size_t blockCount, int M, int N, int K, const skinny_c64* A, int lda,
                     skinny_c64 alpha, const skinny_c64* B, int ldb, skinny_c64 beta, skinny_c64* C,
                     int ldc);
int skinny_tsmttsm_dd(size_t blockCount, int M, int N, int K, const double* A, int lda, double alpha,
                      const double* B, int ldb, double beta, double* C, int ldc);

int skinny_tsmm_s(size_t blockCount, int M, int N, int K, const float* A, int lda, float alpha,
                  const float* B, int ldb, float beta, float* C, int ldc);
int skinny_tsmm_d(size_t blockCount, int M, int N, int K, const double* A, int lda, double alpha,
                  const double* B, int ldb, double beta, double* C, int ldc);
int skinny_tsmm_c(size_t blockCount, int M, int N, int K, const skinny_c32* A, int lda,
                  skinny_c32 alpha, const skinny_c32* B, int ldb, skinny_c32 beta, skinny_c32* C,
                  int ldc);
int skinny_tsmm_z(size_t blockCount, int M, int N, int K, const skinny_c64* A, int lda,
                  skinny_c64 alpha, const skinny_c64* B, int ldb, skinny_c64 beta, skinny_c64* C,
                  int ldc);
int skinny_tsmm_dd(size_t blockCount, int M, int N, int K, const double* A, int lda, double alpha,
                   const double* B, int ldb, double beta, double* C, int ldc);

#ifdef __cplusplus
}
#endif
#endif /* SKINNY_H */
