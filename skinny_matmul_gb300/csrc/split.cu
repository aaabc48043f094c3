// split.cu -- FP64 split-precision products (placeholder until the tensor-core path lands).
#include "api_internal.h"

namespace skinny {
skinny_status split_product(skinny_handle, bool, int64_t, int64_t, int64_t, const double*, int64_t,
                            const void*, const double*, int64_t, const void*, double*, int64_t,
                            cudaStream_t, bool) {
  set_error("split precision: not built");
  return SKINNY_UNSUPPORTED;
}
}  // namespace skinny
