// Mixed-precision kernel instantiations for spin blocks of 2 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE(2, 1, float, f32, true, true, true)
}  // namespace mole
