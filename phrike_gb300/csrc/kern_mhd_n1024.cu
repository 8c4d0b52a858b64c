// 2D MHD x pass and Helmholtz projection instantiations for pencils of 1024 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_MHD_LAUNCHERS(1024)
}  // namespace ps
