// Pass-kernel instantiations for pencils of 1024 points: x, operator and y
// passes (the other groups are in kern_step1d_n1024.cu, kern_last_n1024.cu and
// kern_mhd_n1024.cu, compiled in parallel).
#include "launch.cuh"

namespace ps {
PS_DEFINE_LAUNCHERS(1024)
}  // namespace ps
