// Last-pass instantiations for pencils of 256 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_LAST_LAUNCHERS(256)
}  // namespace ps
