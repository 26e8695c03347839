// FP64 Coriolis kernel instantiations: groups of 33 to 48 blocks, complex64 storage (mixed form).
#include "qd_coriolis64.cuh"

namespace qd {
QD_CORIOLIS_N(48, float2);
}  // namespace qd
