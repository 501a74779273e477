// FP64 instantiation of the spectral passes.
#include "spectral_launch.cuh"

namespace musg {
MUSG_INSTANTIATE_SPECTRAL(double)
}  // namespace musg
