// Pass-kernel instantiations for pencils of 128 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_ALL_LAUNCHERS(128)
}  // namespace ps
