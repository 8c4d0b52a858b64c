// 2D MHD x pass and Helmholtz projection instantiations for pencils of 512 points.
#include "launch.cuh"

namespace ps {
PS_DEFINE_MHD_LAUNCHERS(512)
}  // namespace ps
