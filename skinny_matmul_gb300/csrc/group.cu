// group.cu -- grouped persistent launches: many small TSMTTSM / TSMM problems of one dtype in one
// launch (no counterpart in the reference, whose drivers launch one product at a time on the
// legacy stream, test.cu:114-143, perf.cu:64-96).
//
// Small problems cannot fill 152 SMs on their own: a launch of a K = 2^14, 8 x 8 product streams
// 2 MB in well under the launch and tail time.  Here one persistent launch covers the whole batch:
//   * each problem's K rows are cut into units of about 128 KB of cost, a row's cost being the
//     larger of its operand bytes and its FMAs priced at the dtype's HBM-to-FMA rate ratio (an
//     FP64 64 x 64 row costs ~45x its bytes); a TSMTTSM keeps at most 64 units so that its
//     reduction stays short.  CTA b of G takes the units whose starting cost lies in
//     [b*C/G, (b+1)*C/G) of the class's total cost C (integer costs, so every unit has exactly
//     one owner): a contiguous run with about the same work per CTA;
//   * a CTA finds its first problem by a 32-way search over the descriptors' starting costs (warp
//     0, ballots), then walks forward;
//   * TSMTTSM unit: rows stream through two 32 KB shared buffers with cp.async (double
//     buffering), every thread owns a TT x TT register tile of C for a row slice (TT from
//     min(M, N), at most 8 for FP32 and 4 otherwise), the CTA reduces its tiles in a fixed order into the unit's partial slot, and the
//     last unit to take the problem's ticket sums the unit partials in unit order and applies
//     alpha / beta -- deterministic, and independent of what else is in the batch;
//   * TSMM unit: B staged in shared memory as Bs[m][n], one row per group of lanes, TN outputs per
//     lane, in-place safe (the row is read before the warp passes __syncwarp, then written) --
//     the same arithmetic order as tsmm_kernel, so its results equal the single-problem kernel's.
// No waits on other CTAs: the ticket is a plain atomic and nobody spins.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>

#include "api_internal.h"
#include "group.h"

namespace skinny {

namespace {

constexpr int GT = GROUP_THREADS;
constexpr int64_t UNIT_BYTES = 128 * 1024;  // cost of a unit (bytes-equivalent)
constexpr int64_t UNIT_OVERHEAD = 4096;      // fixed cost per unit in the balance

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
template <int B>
__device__ __forceinline__ void cp_async_ca(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)), "l"(src), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

template <typename T>
__device__ __forceinline__ T scal(const double* v);
template <>
__device__ __forceinline__ float scal<float>(const double* v) {
  return (float)v[0];
}
template <>
__device__ __forceinline__ double scal<double>(const double* v) {
  return v[0];
}
template <>
__device__ __forceinline__ c32 scal<c32>(const double* v) {
  return {(float)v[0], (float)v[1]};
}
template <>
__device__ __forceinline__ c64 scal<c64>(const double* v) {
  return {v[0], v[1]};
}

// rows x cols elements of a row-major operand (leading dimension ld) into a dense shared tile:
// 16-byte copies when the rows are contiguous and aligned, element copies otherwise
template <typename T>
__device__ __forceinline__ void stage_rows(T* dst, const T* src, int64_t ld, int cols, int rows) {
  const int n = rows * cols;
  if (ld == cols && ((reinterpret_cast<uintptr_t>(src) | (uintptr_t)((size_t)n * sizeof(T))) & 15) == 0) {
    const int chunks = (int)((size_t)n * sizeof(T) / 16);
    for (int c = threadIdx.x; c < chunks; c += GT)
      cp_async16(reinterpret_cast<char*>(dst) + 16 * (size_t)c, reinterpret_cast<const char*>(src) + 16 * (size_t)c);
  } else {
    for (int e = threadIdx.x; e < n; e += GT) {
      const int r = e / cols, c = e - r * cols;
      cp_async_ca<(int)sizeof(T)>(dst + e, src + (int64_t)r * ld + c);
    }
  }
}

// TT consecutive values of a shared-memory tile row starting at column c0 (zero past `cols`):
// 16-byte loads where the slice is whole and aligned (4x fewer shared-memory wavefronts than
// scalar loads for FP32 rows of 8), scalar loads otherwise
template <typename T, int TT>
__device__ __forceinline__ void row_slice(const T* row, int c0, int cols, T (&x)[TT]) {
  constexpr int VEC = sizeof(T) < 16 ? 16 / (int)sizeof(T) : 1;
  if constexpr (VEC > 1 && TT % VEC == 0) {
    if (c0 + TT <= cols && (reinterpret_cast<uintptr_t>(row + c0) & 15) == 0) {
#pragma unroll
      for (int v = 0; v < TT / VEC; v++) {
        const uint4 w = *reinterpret_cast<const uint4*>(row + c0 + v * VEC);
        const T* e = reinterpret_cast<const T*>(&w);
#pragma unroll
        for (int k = 0; k < VEC; k++) x[v * VEC + k] = e[k];
      }
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < TT; k++) x[k] = (c0 + k < cols) ? row[c0 + k] : tzero<T>();
}

template <typename T, typename Acc, int TT>
__device__ void tsmttsm_unit(const GroupDesc& g, int64_t ul, unsigned char* smem, unsigned char* partials,
                             unsigned* counter, int* s_last) {
  typedef Ops<T, Acc> O;
  const int tid = threadIdx.x;
  const int M = g.M, N = g.N, code = g.code;
  const bool gram = (code & GF_GRAM) != 0;
  const T* A = static_cast<const T*>(g.A);
  const T* B = static_cast<const T*>(g.B);
  const int64_t lda = g.lda, ldb = g.ldb;
  const int gm = (M + TT - 1) / TT, gn = (N + TT - 1) / TT;
  const int G = gm * gn, RS = GT / G;
  const int cell = tid % G, rs = tid / G;
  const bool active = rs < RS;
  const int m0 = (cell % gm) * TT, n0 = (cell / gm) * TT;
  const int64_t rb = ul * g.rows, re = min(g.K, rb + g.rows);
  const int TR = code >> 8;
  const int boff = gram ? 0 : (int)((TR * M * (int)sizeof(T) + 15) & ~15);
  auto As = [&](int b) { return reinterpret_cast<T*>(smem + b * GROUP_TILE); };
  auto Bs = [&](int b) { return gram ? As(b) : reinterpret_cast<T*>(smem + b * GROUP_TILE + boff); };
  const int ntile = (int)((re - rb + TR - 1) / TR);
  auto issue = [&](int i) {
    const int64_t r0 = rb + (int64_t)i * TR;
    const int rows = (int)min((int64_t)TR, re - r0);
    stage_rows<T>(As(i & 1), A + r0 * lda, lda, M, rows);
    if (!gram) stage_rows<T>(Bs(i & 1), B + r0 * ldb, ldb, N, rows);
    cp_commit();
  };

  Acc acc[TT][TT];
#pragma unroll
  for (int x = 0; x < TT; x++)
#pragma unroll
    for (int y = 0; y < TT; y++) acc[x][y] = O::zero();
  if (ntile > 0) issue(0);
  for (int i = 0; i < ntile; i++) {
    if (i + 1 < ntile) {  // buffer (i+1)&1 was released by the barrier that ended step i-1
      issue(i + 1);
      cp_wait<1>();
    } else {
      cp_wait<0>();
    }
    __syncthreads();
    const int rows = (int)min((int64_t)TR, re - (rb + (int64_t)i * TR));
    const T* as = As(i & 1);
    const T* bs = Bs(i & 1);
    if (active) {
      for (int r = rs; r < rows; r += RS) {
        T a[TT], b[TT];
        row_slice<T, TT>(as + r * M, m0, M, a);
        row_slice<T, TT>(bs + r * N, n0, N, b);
#pragma unroll
        for (int x = 0; x < TT; x++)
#pragma unroll
          for (int y = 0; y < TT; y++) acc[x][y] = O::mac(acc[x][y], a[x], b[y]);
      }
    }
    __syncthreads();
  }

  // ---- CTA reduction in a fixed order into this unit's partial slot --------------------------
  const int MN = M * N;
  Acc* slot = reinterpret_cast<Acc*>(partials + g.part) + (size_t)ul * MN;
  const bool in_smem = (size_t)MN * sizeof(Acc) <= (size_t)GROUP_SMEM;
  Acc* red = in_smem ? reinterpret_cast<Acc*>(smem) : slot;
  int nslots, my_slot;
  bool holder;
  if (32 % G == 0) {
#pragma unroll
    for (int x = 0; x < TT; x++)
#pragma unroll
      for (int y = 0; y < TT; y++)
        for (int o = G; o < 32; o <<= 1) acc[x][y] = O::add(acc[x][y], O::shfl_xor(acc[x][y], o));
    nslots = GT / 32;
    my_slot = tid / 32;
    holder = (tid % 32) < G;
  } else {
    nslots = RS;
    my_slot = rs;
    holder = active;
  }
  for (int sl = 0; sl < nslots; sl++) {
    if (holder && my_slot == sl) {
#pragma unroll
      for (int x = 0; x < TT; x++)
#pragma unroll
        for (int y = 0; y < TT; y++) {
          const int m = m0 + x, n = n0 + y;
          if (m < M && n < N) red[n * M + m] = (sl == 0) ? acc[x][y] : O::add(red[n * M + m], acc[x][y]);
        }
    }
    __syncthreads();
  }
  if (in_smem)
    for (int e = tid; e < MN; e += GT) slot[e] = red[e];
  __threadfence();
  __syncthreads();
  if (tid == 0) *s_last = atomicAdd(counter, 1u) == (unsigned)(g.units - 1);
  __syncthreads();
  if (*s_last) {
    __threadfence();
    const Acc* P = reinterpret_cast<const Acc*>(partials + g.part);
    const T alpha = scal<T>(g.alpha), beta = scal<T>(g.beta);
    const bool bz = (code & GF_BZERO) != 0;
    T* C = static_cast<T*>(g.C);
    const int units = g.units;
    for (int e = tid; e < MN; e += GT) {
      Acc s = O::zero();
      for (int q = 0; q < units; q++) s = O::add(s, ldcg(&P[(size_t)q * MN + e]));
      const int m = e % M, n = e / M;
      T* c = C + (int64_t)n * g.ldc + m;
      *c = O::finish(s, alpha, beta, bz, c);
    }
    if (tid == 0) *counter = 0u;
  }
  __syncthreads();  // shared memory and *s_last are reused by the next unit
}

template <typename T, typename Acc, int TN>
__device__ void tsmm_unit(const GroupDesc& g, int64_t ul, unsigned char* smem) {
  typedef Ops<T, Acc> O;
  const int tid = threadIdx.x;
  const int M = g.M, N = g.N, code = g.code;
  const int gn = code >> 8, np = gn * TN;
  T* Bs = reinterpret_cast<T*>(smem);
  const T* B = static_cast<const T*>(g.B);
  const int64_t ldb = g.ldb;
  const T alpha = scal<T>(g.alpha), beta = scal<T>(g.beta);
  const bool fold = (code & GF_FOLD) != 0;  // the same fold as tsmm_kernel, so the bits agree
  for (int e = tid; e < M * np; e += GT) {
    const int m = e / np, n = e - m * np;
    const T b = (n < N) ? B[(int64_t)n * ldb + m] : tzero<T>();
    Bs[e] = (fold && n < N) ? fold_entry(alpha, b, beta, m == n) : b;
  }
  __syncthreads();
  const T* A = static_cast<const T*>(g.A);
  T* C = static_cast<T*>(g.C);
  const int64_t lda = g.lda, ldc = g.ldc;
  const int RS = GT / gn;
  const int cell = tid % gn, rs = tid / gn;
  const int n0 = cell * TN;
  const bool bz = fold || (code & GF_BZERO) != 0, alpha_one = fold || O::is_one(alpha);
  const int64_t rb = ul * g.rows, re = min(g.K, rb + g.rows);
  for (int64_t base = rb; base < re; base += RS) {  // the same trip count for every lane
    const int64_t r = base + rs;
    const bool valid = r < re;
    Acc acc[TN];
#pragma unroll
    for (int u = 0; u < TN; u++) acc[u] = O::zero();
#pragma unroll 4
    for (int m = 0; m < M; m++) {
      const T a = valid ? A[r * lda + m] : tzero<T>();
      const T* b = Bs + m * np + n0;
#pragma unroll
      for (int u = 0; u < TN; u++) acc[u] = O::mac(acc[u], a, b[u]);
    }
    __syncwarp();  // the row is read by all its lanes before any of it is overwritten (in place)
    if (valid) {
      T* c_row = C + r * ldc;
#pragma unroll
      for (int u = 0; u < TN; u++) {
        const int n = n0 + u;
        if (n < N) {
          const T cv = bz ? tzero<T>() : c_row[n];
          c_row[n] = alpha_one ? O::finish1(acc[u], beta, bz, &cv) : O::finish(acc[u], alpha, beta, bz, &cv);
        }
      }
    }
  }
  __syncthreads();  // Bs is reused by the next unit
}

template <typename T, typename Acc>
__global__ void __launch_bounds__(GT, 2)
    group_kernel(const unsigned char* __restrict__ batch, int cls, unsigned char* partials, unsigned* counters) {
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ GroupDesc sd;
  __shared__ int s_p, s_k, s_last;
  const GroupHeader* H = reinterpret_cast<const GroupHeader*>(batch);
  const int first = H->first[cls], count = H->count[cls];
  const int64_t C = H->cost[cls];
  const int64_t G = gridDim.x, b = blockIdx.x;
  // this CTA's units: starting cost in [lo, hi)
  const int64_t lo = C * b / G, hi = (b == G - 1) ? INT64_MAX : C * (b + 1) / G;
  if (count <= 0 || lo >= hi) return;
  const GroupDesc* D = reinterpret_cast<const GroupDesc*>(batch + sizeof(GroupHeader)) + first;
  const int tid = threadIdx.x;
  if (tid < 32) {  // largest p with D[p].cost0 <= lo (cost0 is non-decreasing, D[0].cost0 == 0)
    const int lane = tid;
    int plo = 0, phi = count;
    while (phi - plo > 1) {
      const int step = (phi - plo + 31) / 32;
      const int cand = plo + lane * step;
      const bool le = cand < phi && D[cand].cost0 <= lo;
      const unsigned m = __ballot_sync(0xffffffffu, le);
      plo += (31 - __clz((int)m)) * step;
      phi = min(phi, plo + step);
    }
    if (lane == 0) {  // first unit of problem plo starting at or after lo
      int p = plo;
      const int64_t c0 = D[p].cost0, uc = D[p].ucost;
      int64_t k = lo > c0 ? (lo - c0 + uc - 1) / uc : 0;
      if (k >= D[p].units) {
        p++;
        k = 0;
      }
      const bool run = p < count && D[p].cost0 + k * D[p].ucost < hi;
      s_p = run ? p : -1;
      s_k = (int)k;
    }
  }
  __syncthreads();
  int loaded = -1;
  for (;;) {
    const int p = s_p, k = s_k;
    if (p < 0) break;
    if (p != loaded) {
      for (int w = tid; w < (int)(sizeof(GroupDesc) / 4); w += GT)
        reinterpret_cast<uint32_t*>(&sd)[w] = reinterpret_cast<const uint32_t*>(D + p)[w];
      __syncthreads();
      loaded = p;
    }
    const int code = sd.code, tl = (code >> 4) & 15;
    if (code & GF_TSMM) {
      switch (tl) {
        case 0: tsmm_unit<T, Acc, 1>(sd, k, smem); break;
        case 1: tsmm_unit<T, Acc, 2>(sd, k, smem); break;
        case 2: tsmm_unit<T, Acc, 4>(sd, k, smem); break;
        default:
          if constexpr (sizeof(Acc) <= 8) tsmm_unit<T, Acc, 8>(sd, k, smem);
          break;
      }
    } else {
      unsigned* ctr = counters + first + p;
      switch (tl) {
        case 0: tsmttsm_unit<T, Acc, 1>(sd, k, smem, partials, ctr, &s_last); break;
        case 1: tsmttsm_unit<T, Acc, 2>(sd, k, smem, partials, ctr, &s_last); break;
        case 2: tsmttsm_unit<T, Acc, 4>(sd, k, smem, partials, ctr, &s_last); break;
        default:
          if constexpr (sizeof(Acc) <= 4) tsmttsm_unit<T, Acc, 8>(sd, k, smem, partials, ctr, &s_last);
          break;
      }
    }
    // every unit ends with a barrier; the next unit (and the stop test) is decided by thread 0
    if (tid == 0) {
      int np = p, nk = k + 1;
      int64_t start;
      if (nk < sd.units) {
        start = sd.cost0 + (int64_t)nk * sd.ucost;
      } else {
        np = p + 1;
        nk = 0;
        start = np < count ? D[np].cost0 : INT64_MAX;
      }
      s_p = (np < count && start < hi) ? np : -1;
      s_k = nk;
    }
    __syncthreads();
  }
}

int ilog2(int v) {
  int l = 0;
  while ((1 << (l + 1)) <= v) l++;
  return l;
}

}  // namespace

void* group_kernel_fn(int cls) {
  static SmemAttr attr[GROUP_CLASSES];  // the shared-memory attribute, per class and device
  void* fn = nullptr;
  switch (cls) {
    case SKINNY_R32: fn = (void*)group_kernel<float, float>; break;
    case SKINNY_R64: fn = (void*)group_kernel<double, double>; break;
    case SKINNY_C32: fn = (void*)group_kernel<c32, c32>; break;
    case SKINNY_C64: fn = (void*)group_kernel<c64, c64>; break;
    default: return nullptr;
  }
  if (!ensure_smem_attr(fn, GROUP_SMEM, attr[cls])) return nullptr;
  return fn;
}

int group_grid(int sms) { return 2 * sms; }

// FMAs of the dtype worth one byte of HBM traffic: GB300 streams 6707 GB/s and retires 595 G FP64
// FMAs/s (complex FP64: 4 FMAs per product) and 37 T FP32 FMAs/s, so FP64 products cost ~11
// bytes-equivalent per FMA and FP32 products are priced by their bytes.
static double fma_bytes(skinny_dtype dt) { return (dt == SKINNY_R64 || dt == SKINNY_C64) ? 11.3 : 0.18; }
static int64_t fmas_per_product(skinny_dtype dt) { return (dt == SKINNY_C32 || dt == SKINNY_C64) ? 4 : 1; }

// row cost (bytes-equivalent) and row bytes of an item
static void row_cost(const skinny_group_item& it, skinny_dtype dt, int64_t* bytes, int64_t* cost) {
  const int64_t es = (int64_t)dtype_size(dt);
  const bool bz = it.beta[0] == 0.0 && it.beta[1] == 0.0;
  int64_t rb, fma;
  if (it.op == SKINNY_OP_TSMM) {
    const bool inplace = it.A == (const void*)it.C;
    rb = (it.M + (bz || inplace ? 1 : 2) * it.N) * es;
    fma = (it.M * it.N + it.N) * fmas_per_product(dt);
  } else {
    const bool gram = it.A == it.B && it.lda == it.ldb && it.M == it.N;
    rb = (it.M + (gram ? 0 : it.N)) * es;
    fma = it.M * it.N * fmas_per_product(dt);
  }
  *bytes = rb;
  *cost = std::max<int64_t>(rb, (int64_t)std::ceil((double)fma * fma_bytes(dt)));
}

double group_item_cost(const skinny_group_item& it, skinny_dtype dt) {
  int64_t rb, rc;
  row_cost(it, dt, &rb, &rc);
  return (double)rc * (double)it.K;
}

skinny_status group_plan(const skinny_group_item* items, const skinny_dtype* dts, int n,
                         std::vector<unsigned char>& out, size_t* part_bytes, std::vector<int>* order) {
  if (n < 0 || (n > 0 && (!items || !dts))) {
    set_error("group: bad item list");
    return SKINNY_BAD_ARG;
  }
  GroupHeader hd;
  std::memset(&hd, 0, sizeof hd);
  std::vector<GroupDesc> descs;
  std::vector<int> ord;
  descs.reserve(n);
  size_t part = 0;
  for (int cls = 0; cls < GROUP_CLASSES; cls++) {
    hd.first[cls] = (int32_t)descs.size();
    int64_t cost_cls = 0;
    for (int i = 0; i < n; i++) {
      if ((int)dts[i] != cls) continue;
      const skinny_group_item& it = items[i];
      const skinny_dtype dt = dts[i];
      const bool tsmm = it.op == SKINNY_OP_TSMM;
      if (it.op != SKINNY_OP_TSMM && it.op != SKINNY_OP_TSMTTSM) {
        set_error("group: item " + std::to_string(i) + " is neither TSMTTSM nor TSMM");
        return SKINNY_BAD_ARG;
      }
      skinny_status s = check_args(tsmm, dt, it.M, it.N, it.K, it.A, it.lda, it.alpha, it.B, it.ldb, it.beta, it.C,
                                   it.ldc);
      if (s != SKINNY_OK) return s;
      if (it.M > GROUP_MAX_W || it.N > GROUP_MAX_W) {
        set_error("group: M, N <= 64 for a grouped item");
        return SKINNY_UNSUPPORTED;
      }
      const size_t es = dtype_size(dt), al = es;  // natural alignment of the element type
      if ((uintptr_t)it.A % al || (uintptr_t)it.B % al || (uintptr_t)it.C % al) {
        set_error("group: operands must be aligned to their element size");
        return SKINNY_BAD_ARG;
      }
      if (it.M == 0 || it.N == 0 || (tsmm && it.K == 0)) continue;  // nothing to compute
      const bool bz = it.beta[0] == 0.0 && it.beta[1] == 0.0;
      // register tiles within 128 registers (two CTAs per SM): TSMTTSM 8 x 8 for FP32 only,
      // 4 x 4 otherwise; TSMM up to 8 outputs per lane (4 for complex FP64)
      const int cap_t = es <= 4 ? 8 : 4, cap_n = es <= 8 ? 8 : 4;
      int64_t rb, rc;
      row_cost(it, dt, &rb, &rc);
      GroupDesc d;
      std::memset(&d, 0, sizeof d);
      d.A = it.A;
      d.B = it.B;
      d.C = it.C;
      d.K = it.K;
      d.lda = it.lda;
      d.ldb = it.ldb;
      d.ldc = it.ldc;
      std::memcpy(d.alpha, it.alpha, sizeof d.alpha);
      std::memcpy(d.beta, it.beta, sizeof d.beta);
      d.M = (int32_t)it.M;
      d.N = (int32_t)it.N;
      int code = bz ? GF_BZERO : 0;
      int64_t rows, units;
      if (tsmm) {
        const int tn = std::min(pow2ceil(it.N), cap_n);
        const int gn = pow2ceil((it.N + tn - 1) / tn);
        const int RS = GROUP_THREADS / gn;
        rows = round_up(std::max<int64_t>(RS, UNIT_BYTES / rc), RS);
        units = (it.K + rows - 1) / rows;
        code |= GF_TSMM | (ilog2(tn) << 4) | (gn << 8);
        if (it.A == it.C && it.lda == it.ldc && it.M == it.N && !bz) code |= GF_FOLD;
      } else {
        const bool gram = it.A == it.B && it.lda == it.ldb && it.M == it.N;
        const int tt = std::min(pow2ceil(std::min(it.M, it.N)), cap_t);
        const int tr = (int)((GROUP_TILE - 16) / rb);
        const int64_t MN = it.M * it.N;
        // at most 64 units, and their partials at most ~1 MB, so the closing sum stays short
        const int64_t ucap = std::max<int64_t>(1, std::min<int64_t>(64, ((int64_t)1 << 20) / (MN * (int64_t)es)));
        units = std::max<int64_t>(1, (it.K * rc + UNIT_BYTES - 1) / UNIT_BYTES);
        units = std::min(units, ucap);
        rows = (it.K + units - 1) / units;
        if (rows > 0) units = (it.K + rows - 1) / rows;
        d.part = (int64_t)part;
        part += (size_t)round_up(units * MN * (int64_t)es, 256);
        code |= (gram ? GF_GRAM : 0) | (ilog2(tt) << 4) | (tr << 8);
      }
      d.rows = rows;
      d.units = (int32_t)units;
      d.code = code;
      // a unit's cost: its rows, plus a fixed share for staging B / reducing the tile sums
      d.ucost = rows * rc + UNIT_OVERHEAD;
      d.cost0 = cost_cls;
      cost_cls += units * d.ucost;
      descs.push_back(d);
      ord.push_back(i);
    }
    hd.count[cls] = (int32_t)descs.size() - hd.first[cls];
    hd.cost[cls] = cost_cls;
  }
  out.resize(sizeof(GroupHeader) + descs.size() * sizeof(GroupDesc));
  std::memcpy(out.data(), &hd, sizeof hd);
  if (!descs.empty()) std::memcpy(out.data() + sizeof hd, descs.data(), descs.size() * sizeof(GroupDesc));
  if (part_bytes) *part_bytes = part;
  if (order) *order = std::move(ord);
  return SKINNY_OK;
}

}  // namespace skinny

using namespace skinny;

// Per-(handle, stream) buffers of skinny_group: the batch, the unit partials, the tickets.
struct GroupWs {
  unsigned char* batch = nullptr;
  size_t batch_cap = 0;
  unsigned char* part = nullptr;
  size_t part_cap = 0;
  unsigned* counters = nullptr;
  size_t counters_cap = 0;
};

static std::mutex g_group_mu;
static std::map<std::pair<skinny_handle, cudaStream_t>, GroupWs> g_group_ws;

static skinny_status grow(void** p, size_t* cap, size_t need, cudaStream_t st, bool zero) {
  if (need <= *cap) return SKINNY_OK;
  if (*p) {
    cudaStreamSynchronize(st);  // earlier batches on this stream may still use the old buffer
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
  }
  size_t nb = std::max<size_t>(need + need / 2, 1 << 16);
  if (cudaMalloc(p, nb) != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    set_error("group: cudaMalloc failed");
    return SKINNY_NO_MEM;
  }
  if (zero && cudaMemsetAsync(*p, 0, nb, st) != cudaSuccess) {
    set_error("group: cudaMemsetAsync failed");
    return SKINNY_DEVICE_ERROR;
  }
  *cap = nb;
  return SKINNY_OK;
}

extern "C" skinny_status skinny_group(skinny_handle h, skinny_dtype dtype, const skinny_group_item* items,
                                      int32_t count, void* stream) {
  if (!h || count < 0 || (count > 0 && !items) || dtype_size(dtype) == 0) {
    set_error("group: bad arguments");
    return SKINNY_BAD_ARG;
  }
  if (count == 0) return SKINNY_OK;
  std::vector<skinny_dtype> dts((size_t)count, dtype);
  std::vector<unsigned char> batch;
  size_t part_bytes = 0;
  skinny_status s = group_plan(items, dts.data(), count, batch, &part_bytes, nullptr);
  if (s != SKINNY_OK) return s;
  const GroupHeader* hd = reinterpret_cast<const GroupHeader*>(batch.data());
  if (hd->count[dtype] == 0) return SKINNY_OK;
  DevGuard g(h->dev.id);
  cudaStream_t st = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_group_mu);
  GroupWs& ws = g_group_ws[std::make_pair(h, st)];
  if ((s = grow((void**)&ws.batch, &ws.batch_cap, batch.size(), st, false)) != SKINNY_OK) return s;
  if ((s = grow((void**)&ws.part, &ws.part_cap, std::max<size_t>(part_bytes, 256), st, false)) != SKINNY_OK) return s;
  if ((s = grow((void**)&ws.counters, &ws.counters_cap, (size_t)count * sizeof(unsigned), st, true)) != SKINNY_OK)
    return s;
  // pageable source: the copy is staged before the call returns, so `batch` may go out of scope
  if (cudaMemcpyAsync(ws.batch, batch.data(), batch.size(), cudaMemcpyHostToDevice, st) != cudaSuccess) {
    set_error("group: descriptor upload failed");
    return SKINNY_DEVICE_ERROR;
  }
  void* fn = group_kernel_fn(dtype);
  if (!fn) return SKINNY_DEVICE_ERROR;
  const unsigned char* b = ws.batch;
  int cls = (int)dtype;
  void* args[] = {(void*)&b, (void*)&cls, (void*)&ws.part, (void*)&ws.counters};
  cudaError_t e = cudaLaunchKernel(fn, dim3(group_grid(h->dev.sms)), dim3(GROUP_THREADS), args, GROUP_SMEM, st);
  count_launch();
  if (e != cudaSuccess) {
    cudaGetLastError();
    set_error(std::string("group launch: ") + cudaGetErrorString(e));
    return SKINNY_DEVICE_ERROR;
  }
  return SKINNY_OK;
}

// Frees the skinny_group buffers of a handle (called by skinny_destroy).
namespace skinny {
void group_release(skinny_handle h) {
  std::lock_guard<std::mutex> lk(g_group_mu);
  for (auto it = g_group_ws.begin(); it != g_group_ws.end();) {
    if (it->first.first == h) {
      cudaFree(it->second.batch);
      cudaFree(it->second.part);
      cudaFree(it->second.counters);
      it = g_group_ws.erase(it);
    } else {
      ++it;
    }
  }
}
}  // namespace skinny
