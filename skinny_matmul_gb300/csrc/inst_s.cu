// inst_s.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for storage type
// float with accumulator float (one translation unit per type pair, so that the build runs in
// parallel).
#include "launch.cuh"

namespace skinny {
SKINNY_LAUNCHERS(, float, float)
}  // namespace skinny
