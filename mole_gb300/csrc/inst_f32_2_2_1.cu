// Mixed-precision VMC launchers with two-parameter SR sums, spin blocks of 2 up and 2 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_VMC(2, 2, float, f32, 1, 2)
}  // namespace mole
