// FP64 Coriolis kernel instantiations: groups of 25 to 32 blocks, complex128 and complex64 storage.
#include "qd_coriolis64.cuh"

namespace qd {
QD_CORIOLIS_N(32, double2);
QD_CORIOLIS_N(32, float2);
}  // namespace qd
