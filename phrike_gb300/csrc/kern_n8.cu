// Pass-kernel instantiations for pencils of 8 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_ALL_LAUNCHERS(8)
}  // namespace ps
