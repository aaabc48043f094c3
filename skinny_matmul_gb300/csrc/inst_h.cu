// inst_h.cu -- explicit instantiation of the CUDA-core TSMTTSM launcher for C = alpha A^H B + beta C
// (complex, left operand conjugated): storage/accumulator types c32h and c64h.
#include "launch.cuh"

namespace skinny {
template skinny_status tsmttsm_run<c32h, c32h>(const DeviceInfo&, Workspace&, int*, cudaStream_t, int64_t,
                                            int64_t, int64_t, const c32h*, int64_t, c32h, const c32h*,
                                            int64_t, c32h, bool, c32h*, int64_t, const LaunchOpts&);
template skinny_status tsmttsm_run<c64h, c64h>(const DeviceInfo&, Workspace&, int*, cudaStream_t, int64_t,
                                            int64_t, int64_t, const c64h*, int64_t, c64h, const c64h*,
                                            int64_t, c64h, bool, c64h*, int64_t, const LaunchOpts&);
}  // namespace skinny
