// FP64 kernel instantiations for spin blocks of 2 up and 2 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE(2, 2, double, f64, true, true, true)
}  // namespace mole
