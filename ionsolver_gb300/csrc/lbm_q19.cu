// lbm_q19.cu -- instantiates the timestep kernels for the D3Q19 velocity set.
#include "lbm_kernels.cuh"

namespace ion {
ION_DEFINE_LBM_DISPATCH(19, q19)
}  // namespace ion
