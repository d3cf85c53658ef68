// lbm_q19.cu -- instantiates the timestep kernels for the D3Q19 velocity set.  The
// stream_collide kernels of each storage type are instantiated in their own
// translation unit (lbm_q19_sc.cu, compiled once per type) so they build in parallel.
#include "lbm_kernels.cuh"

namespace ion {
extern template void launch_sc<19, ION_FP32>(const DevLbm&, int, bool, uint32_t, unsigned, uint32_t*, cudaStream_t);
extern template void launch_sc<19, ION_FP16S>(const DevLbm&, int, bool, uint32_t, unsigned, uint32_t*, cudaStream_t);
extern template void launch_sc<19, ION_FP16C>(const DevLbm&, int, bool, uint32_t, unsigned, uint32_t*, cudaStream_t);
ION_DEFINE_LBM_DISPATCH(19, q19)
}  // namespace ion
