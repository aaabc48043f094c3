// inst_s_dd.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for storage
// type float with accumulator double (the double-double method for FP32) (one translation unit per
// type pair, so that the build runs in parallel).
#include "launch.cuh"

namespace skinny {
SKINNY_LAUNCHERS(, float, double)
}  // namespace skinny
