// FP64 evaluation and DMC launchers, spin blocks of 1 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_PART_REST(1, 1, double, f64)
}  // namespace mole
