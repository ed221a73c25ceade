// Mixed-precision evaluation and DMC launchers, spin blocks of 2 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_REST(2, 1, float, f32)
}  // namespace mole
