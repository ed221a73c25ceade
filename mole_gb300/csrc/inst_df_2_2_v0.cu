// Double-float (FP64-accurate) VMC launchers without the e-n Jastrow, spin blocks of 2 up and 2 down electrons.
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE_DF_VMC(2, 2, 0)
}  // namespace mole
