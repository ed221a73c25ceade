// Mixed-precision VMC launchers with eight-wide SR sums, spin blocks of 2 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_VMC(2, 1, float, f32, 2, 8)
}  // namespace mole
