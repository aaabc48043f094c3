// svqb.cu -- on-device SVQB (placeholder).
#include "api_internal.h"
extern "C" skinny_status skinny_svqb(skinny_handle, skinny_acc, int64_t, int64_t, double*, int64_t,
                                     double*, void*) {
  skinny::set_error("svqb: not built");
  return SKINNY_UNSUPPORTED;
}
