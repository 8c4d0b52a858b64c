// Pass-kernel instantiations for pencils of 512 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_LAUNCHERS(512)
}  // namespace ps
