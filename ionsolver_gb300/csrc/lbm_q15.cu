// lbm_q15.cu -- instantiates the timestep kernels for the D3Q15 velocity set.
#include "lbm_kernels.cuh"

namespace ion {
ION_DEFINE_LBM_DISPATCH(15, q15)
}  // namespace ion
