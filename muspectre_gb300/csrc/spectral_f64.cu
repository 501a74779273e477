// FP64 instantiation of the spectral passes.
#include "spectral_launch.cuh"

namespace musg {
MUSG_INSTANTIATE_SPECTRAL(double)

int cg_operator_partials(const Spectral &sp) {
  // the last pass has the most blocks in either precision (the FP32 plan packs
  // at least as many rows per block as the FP64 one)
  return last_cfg<double>(sp).blocks;
}
}  // namespace musg
