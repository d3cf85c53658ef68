// lbm_q19_sc.cu -- the D3Q19 stream_collide kernels of one DDF storage type,
// ION_SC_FT (ION_FP32, ION_FP16S or ION_FP16C), given on the compiler's command line.
#include "lbm_kernels.cuh"

#ifndef ION_SC_FT
#error "compile with -DION_SC_FT=<storage type>"
#endif

namespace ion {
template void launch_sc<19, ION_SC_FT>(const DevLbm&, int, bool, uint32_t, unsigned, uint32_t*, cudaStream_t);
}  // namespace ion
