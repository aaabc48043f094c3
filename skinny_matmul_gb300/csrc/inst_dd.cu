// inst_dd.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for storage type
// double with accumulator dd (the double-double method) (one translation unit per type pair, so
// that the build runs in parallel).
#include "launch.cuh"

namespace skinny {
SKINNY_LAUNCHERS(, double, dd)
}  // namespace skinny
