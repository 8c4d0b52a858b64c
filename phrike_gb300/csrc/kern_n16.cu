// Pass-kernel instantiations for pencils of 16 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_ALL_LAUNCHERS(16)
}  // namespace ps
