// 1D whole-step kernel instantiations for pencils of 1024 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_STEP1D_LAUNCHERS(1024)
}  // namespace ps
