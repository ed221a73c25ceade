// FP64 VMC launchers with eight-wide SR sums, spin blocks of 1 up and 0 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_VMC(1, 0, double, f64, 2, 8)
}  // namespace mole
