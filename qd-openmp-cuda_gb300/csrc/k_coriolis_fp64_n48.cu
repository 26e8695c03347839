// FP64 Coriolis kernel instantiations: groups of 33 to 48 blocks, complex128 storage.
#include "qd_coriolis64.cuh"

namespace qd {
QD_CORIOLIS_N(48, double2);
}  // namespace qd
