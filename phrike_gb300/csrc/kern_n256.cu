// Pass-kernel instantiations for pencils of 256 points: x, operator and y
// passes (the other groups are in kern_step1d_n256.cu, kern_last_n256.cu and
// kern_mhd_n256.cu, compiled in parallel).
#include "launch.cuh"

namespace ps {
PS_DEFINE_LAUNCHERS(256)
}  // namespace ps
