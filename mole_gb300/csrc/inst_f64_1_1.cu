// FP64 kernel instantiations for spin blocks of 1 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE(1, 1, double, f64, true, true, true)
}  // namespace mole
