// FP32-form neural-Jastrow kernel instantiations for 2 up and 2 down electrons (LiH, Be).
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE_NN(2, 2, float, f32)
}  // namespace mole
