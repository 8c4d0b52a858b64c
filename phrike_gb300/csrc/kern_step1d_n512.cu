// 1D whole-step kernel instantiations for pencils of 512 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_STEP1D_LAUNCHERS(512)
}  // namespace ps
