// Mixed-precision VMC launchers with eight-wide SR sums, spin blocks of 2 up and 2 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_VMC(2, 2, float, f32, 2, 8)
}  // namespace mole
