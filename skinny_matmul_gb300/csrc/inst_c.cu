// inst_c.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for
// storage type c32 with accumulator c32 (one translation unit per type so the build runs in parallel).
#include "launch.cuh"

namespace skinny {
template skinny_status tsmttsm_run<c32, c32>(const DeviceInfo&, Workspace&, int*, cudaStream_t, int64_t,
                                          int64_t, int64_t, const c32*, int64_t, c32, const c32*,
                                          int64_t, c32, bool, c32*, int64_t, const LaunchOpts&);
template skinny_status tsmm_run<c32, c32>(const DeviceInfo&, cudaStream_t, int64_t, int64_t, int64_t,
                                       const c32*, int64_t, c32, const c32*, int64_t, c32, bool, c32*,
                                       int64_t, const LaunchOpts&);
}  // namespace skinny
