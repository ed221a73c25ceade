// Mixed-precision VMC launchers without SR sums, spin blocks of 2 up and 2 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_VMC(2, 2, float, f32, 0, 0)
}  // namespace mole
