// 1D-only pencil length 2048: the whole-step kernel and the contiguous operator.
#include "launch.cuh"

namespace ps {
PS_DEFINE_LAUNCHERS_1D(2048)
}  // namespace ps
