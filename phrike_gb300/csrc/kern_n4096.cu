// 1D-only pencil length 4096: the whole-step kernel and the contiguous operator.
#include "launch.cuh"

namespace ps {
PS_DEFINE_LAUNCHERS_1D(4096)
}  // namespace ps
