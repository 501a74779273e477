// FP64 instantiation of the spectral passes.
#include "spectral_launch.cuh"

namespace musg {
MUSG_INSTANTIATE_SPECTRAL(double)

void grouped_op_destroy(GroupedOp *op) { delete op; }
int grouped_op_fwd_partials(const GroupedOp *op, int b) { return op->fwd_parts[b]; }
}  // namespace musg
