// inst_z_dd.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for storage
// type c64 with accumulator zdd (the double-double method for complex FP64) (one translation unit
// per type pair, so that the build runs in parallel).
#include "launch.cuh"

namespace skinny {
SKINNY_LAUNCHERS(, c64, zdd)
}  // namespace skinny
