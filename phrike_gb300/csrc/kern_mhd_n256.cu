// 2D MHD x pass and Helmholtz projection instantiations for pencils of 256 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_MHD_LAUNCHERS(256)
}  // namespace ps
