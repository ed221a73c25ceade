// FP64 VMC launchers without SR sums, spin blocks of 1 up and 0 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_VMC(1, 0, double, f64, 0, 0)
}  // namespace mole
