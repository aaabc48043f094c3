// inst_c_dd.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for storage
// type c32 with accumulator c64 (the double-double method for complex FP32) (one translation unit
// per type pair, so that the build runs in parallel).
#include "launch.cuh"

namespace skinny {
SKINNY_LAUNCHERS(, c32, c64)
}  // namespace skinny
