// FP64 neural-Jastrow kernel instantiations for 2 up and 2 down electrons (LiH, Be).
#include "dispatch.cuh"

namespace mole {
MOLE_INSTANTIATE_NN(2, 2, double, f64)
}  // namespace mole
