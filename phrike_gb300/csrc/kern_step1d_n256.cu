// 1D whole-step kernel instantiations for pencils of 256 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_STEP1D_LAUNCHERS(256)
}  // namespace ps
