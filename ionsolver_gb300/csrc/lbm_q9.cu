// lbm_q9.cu -- instantiates the timestep kernels for the D2Q9 velocity set.
#include "lbm_kernels.cuh"

namespace ion {
ION_DEFINE_LBM_DISPATCH(9, q9)
}  // namespace ion
