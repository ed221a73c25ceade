// Mixed-precision VMC launchers without SR sums, spin blocks of 2 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_VMC(2, 1, float, f32, 0, 0)
}  // namespace mole
