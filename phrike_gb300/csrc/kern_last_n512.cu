// Last-pass instantiations for pencils of 512 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_LAST_LAUNCHERS(512)
}  // namespace ps
