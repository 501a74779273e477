// FP32 instantiation of the spectral passes.
#include "spectral_launch.cuh"

namespace musg {
MUSG_INSTANTIATE_SPECTRAL(float)
}  // namespace musg
