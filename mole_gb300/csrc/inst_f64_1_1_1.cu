// FP64 VMC launchers with two-parameter SR sums, spin blocks of 1 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_VMC(1, 1, double, f64, 1, 2)
}  // namespace mole
