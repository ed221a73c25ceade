// Double-float (FP64-accurate) evaluation launchers, spin blocks of 2 up and 2 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE_DF_EVAL(2, 2)
}  // namespace mole
