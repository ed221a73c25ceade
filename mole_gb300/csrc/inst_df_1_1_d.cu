// Double-float (FP64-accurate) DMC step launchers, spin blocks of 1 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE_DF_DMC(1, 1)
}  // namespace mole
