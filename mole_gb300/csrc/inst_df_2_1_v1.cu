// Double-float (FP64-accurate) VMC launchers with the e-n Jastrow, spin blocks of 2 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE_DF_VMC(2, 1, 1)
}  // namespace mole
