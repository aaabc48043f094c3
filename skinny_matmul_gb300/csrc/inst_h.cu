// inst_h.cu -- explicit instantiation of the CUDA-core TSMTTSM / TSMM launchers for C = alpha A^H
// B + beta C (complex, left operand conjugated): storage/accumulator types c32h and c64h (one
// translation unit per type pair, so that the build runs in parallel).
#include "launch.cuh"

namespace skinny {
SKINNY_LAUNCHERS(, c32h, c32h)
SKINNY_LAUNCHERS(, c64h, c64h)
}  // namespace skinny
