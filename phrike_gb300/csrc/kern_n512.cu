// Pass-kernel instantiations for pencils of 512 points: x, operator and y
// passes (the other groups are in kern_step1d_n512.cu, kern_last_n512.cu and
// kern_mhd_n512.cu, compiled in parallel).
#include "launch.cuh"

namespace ps {
PS_DEFINE_LAUNCHERS(512)
}  // namespace ps
