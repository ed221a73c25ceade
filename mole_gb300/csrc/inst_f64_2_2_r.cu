// FP64 evaluation and DMC launchers, spin blocks of 2 up and 2 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_REST(2, 2, double, f64)
}  // namespace mole
