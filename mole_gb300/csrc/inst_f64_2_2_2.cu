// FP64 VMC launchers with eight-wide SR sums, spin blocks of 2 up and 2 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_VMC(2, 2, double, f64, 2, 8)
}  // namespace mole
