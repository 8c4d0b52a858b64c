// Pass-kernel instantiations for pencils of 32 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_ALL_LAUNCHERS(32)
}  // namespace ps
