// Pass-kernel instantiations for pencils of 64 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_ALL_LAUNCHERS(64)
}  // namespace ps
