// FP64 Coriolis kernel instantiations: groups of at most 2, 4, 8, 16 and 24 blocks.
#include "qd_coriolis64.cuh"

namespace qd {
QD_CORIOLIS_N(2, double2);
QD_CORIOLIS_N(4, double2);
QD_CORIOLIS_N(8, double2);
QD_CORIOLIS_N(16, double2);
QD_CORIOLIS_N(24, double2);
}  // namespace qd
