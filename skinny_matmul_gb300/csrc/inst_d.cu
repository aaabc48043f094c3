// inst_d.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for storage type
// double with accumulator double (one translation unit per type pair, so that the build runs in
// parallel).
#include "launch.cuh"

namespace skinny {
SKINNY_LAUNCHERS(, double, double)
}  // namespace skinny

namespace skinny {
// used by the allocation-free entry point in static_scratch.cu
template skinny_status tsmttsm_plan<double, double>(const DeviceInfo&, int64_t, int64_t, int64_t,
                                                    const void*, int64_t, const void*, int64_t, bool,
                                                    const LaunchOpts&, TsmttsmPlan&);
template skinny_status tsmttsm_dispatch<double, double>(int, int, const TsmttsmArgs<double>&, dim3,
                                                        int, cudaStream_t);
}  // namespace skinny
