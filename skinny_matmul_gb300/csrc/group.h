// group.h -- grouped launches: the batch format shared by group.cu (kernels, planner,
// skinny_group) and serve.cu (the request loop's graph-replayed lane).
//
// A batch in device memory is one GroupHeader followed by GroupDesc[n].  Descriptors are ordered
// by dtype class (class = skinny_dtype value); one kernel per class reads its range.  Each
// problem's rows are cut into `units` units of equal estimated cost (`ucost`, in bytes-equivalent:
// the larger of the unit's operand bytes and its FMAs at the HBM-to-FMA rate ratio of the dtype);
// cost0 is the cost before the problem's first unit within its class, and CTA b of G takes the
// units whose starting cost lies in [b*C/G, (b+1)*C/G), C = the class's total cost -- a
// contiguous run of units with about the same work per CTA.
#pragma once
#include <cstdint>
#include <vector>

#include "skinny.h"

namespace skinny {

constexpr int GROUP_THREADS = 256;
constexpr int GROUP_TILE = 32768;            // bytes of one staging buffer (two per CTA)
constexpr int GROUP_SMEM = 2 * GROUP_TILE;   // dynamic shared memory per CTA
constexpr int GROUP_MAX_W = 64;              // M, N limit of a grouped problem
constexpr int GROUP_CLASSES = 4;             // R32, R64, C32, C64

// GF_FOLD: in-place TSMM with M == N and beta != 0, computed as C = A (alpha B + beta I)
enum : int32_t { GF_TSMM = 1, GF_GRAM = 2, GF_BZERO = 4, GF_FOLD = 8 };

struct GroupHeader {
  int32_t first[GROUP_CLASSES];  // first descriptor of each class
  int32_t count[GROUP_CLASSES];  // descriptors of each class
  int64_t cost[GROUP_CLASSES];   // total cost of each class
  int64_t pad[8];
};
static_assert(sizeof(GroupHeader) == 128, "GroupHeader is 128 bytes");

struct GroupDesc {
  const void* A;
  const void* B;
  void* C;
  int64_t K, lda, ldb, ldc;
  int64_t cost0;  // cost of the class's units before this problem's first unit
  int64_t ucost;  // cost of one unit (> 0)
  int64_t rows;   // rows per unit (the last unit may be shorter)
  int64_t part;   // byte offset of this problem's unit partials (TSMTTSM)
  double alpha[2], beta[2];
  int32_t M, N;
  int32_t units;
  int32_t code;  // bits 0-3 GF_* flags, bits 4-7 log2(register tile), bits 8-31 tile rows (TSMTTSM) or
                 // cells per row (TSMM)
  int64_t pad;
};
static_assert(sizeof(GroupDesc) == 144, "GroupDesc is 144 bytes");

// Plans a batch of items whose dtypes are dts[i]: writes header + descriptors (classes in dtype
// order) to `out`, the byte size of the unit partials to *part_bytes, and maps descriptor d to
// item order[d].  Items with nothing to compute (M or N zero, TSMM with K == 0) are left out.
// Checks every item (layout rules of skinny_tsmttsm / skinny_tsmm, M, N <= 64, natural alignment).
skinny_status group_plan(const skinny_group_item* items, const skinny_dtype* dts, int n,
                         std::vector<unsigned char>& out, size_t* part_bytes, std::vector<int>* order);

// Kernel entry of class c, its persistent grid on this device and its dynamic shared memory;
// sets the kernel's shared-memory attribute on first use.
void* group_kernel_fn(int cls);
int group_grid(int sms);

// Cost of a whole item in bytes-equivalent (the larger of its algorithmic bytes, perf.cu:208-232,
// and its FMAs at the dtype's HBM-to-FMA rate ratio): the request loop's measure of "small".
double group_item_cost(const skinny_group_item& it, skinny_dtype dt);

}  // namespace skinny
