// Mixed-precision kernel instantiations for spin blocks of 2 up and 2 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE(2, 2, float, f32, true, true, true)
}  // namespace mole
