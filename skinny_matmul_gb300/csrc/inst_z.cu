// inst_z.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for
// storage type c64 with accumulator c64 (one translation unit per type so the build runs in parallel).
#include "launch.cuh"

namespace skinny {
template skinny_status tsmttsm_run<c64, c64>(const DeviceInfo&, Workspace&, int*, cudaStream_t, int64_t,
                                          int64_t, int64_t, const c64*, int64_t, c64, const c64*,
                                          int64_t, c64, bool, c64*, int64_t, const LaunchOpts&);
template skinny_status tsmm_run<c64, c64>(const DeviceInfo&, cudaStream_t, int64_t, int64_t, int64_t,
                                       const c64*, int64_t, c64, const c64*, int64_t, c64, bool, c64*,
                                       int64_t, const LaunchOpts&);
}  // namespace skinny
