// inst_z.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for storage type
// c64 with accumulator c64 (one translation unit per type pair, so that the build runs in
// parallel).
#include "launch.cuh"

namespace skinny {
SKINNY_LAUNCHERS(, c64, c64)
}  // namespace skinny
