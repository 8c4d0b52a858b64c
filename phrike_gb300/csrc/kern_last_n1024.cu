// Last-pass instantiations for pencils of 1024 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_LAST_LAUNCHERS(1024)
}  // namespace ps
