// Double-float (FP64-accurate) VMC launchers without the e-n Jastrow, spin blocks of 1 up and 1 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE_DF_VMC(1, 1, 0)
}  // namespace mole
