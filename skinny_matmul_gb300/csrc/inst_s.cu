// inst_s.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for
// storage type float with accumulator float (one translation unit per type so the build runs in parallel).
#include "launch.cuh"

namespace skinny {
template skinny_status tsmttsm_run<float, float>(const DeviceInfo&, Workspace&, int*, cudaStream_t, int64_t,
                                          int64_t, int64_t, const float*, int64_t, float, const float*,
                                          int64_t, float, bool, float*, int64_t, const LaunchOpts&);
template skinny_status tsmm_run<float, float>(const DeviceInfo&, cudaStream_t, int64_t, int64_t, int64_t,
                                       const float*, int64_t, float, const float*, int64_t, float, bool, float*,
                                       int64_t, const LaunchOpts&);
}  // namespace skinny
