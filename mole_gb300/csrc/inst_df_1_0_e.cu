// Double-float (FP64-accurate) evaluation launchers, spin blocks of 1 up and 0 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE_DF_EVAL(1, 0)
}  // namespace mole
