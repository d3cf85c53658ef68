// reduce_f64.cuh -- FP64 sums of stored DDF values, shared by the handle's
// reduction (ion_lbm_mass_charge, setup_kernels.cu) and the allocation-free
// one (ion_ddf_sum_f64_noalloc, noalloc.cu).
//
// Pass 1: block b sums values [b*per, min((b+1)*per, count)) decoded to
// double, each thread a strided sub-sum, then a fixed tree in shared memory.
// Pass 2: one block sums the partials the same way.  The order of additions
// depends only on (count, per, number of blocks), so a sum is reproducible.
#pragma once
#include "ion_device.cuh"
#include "ion_launch.h"

namespace ion {

__device__ __forceinline__ double block_tree_sum(double s, double* sh) {
    sh[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = RED_BLOCK / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    return sh[0];
}

template <int FT>
static __global__ void __launch_bounds__(RED_BLOCK) k_sum_partial(const void* x, uint64_t count, uint64_t per,
                                                                  double* partials) {
    __shared__ double sh[RED_BLOCK];
    const uint64_t b = (uint64_t)blockIdx.x * per, e = min(b + per, count);
    double s = 0.0;
    for (uint64_t i = b + threadIdx.x; i < e; i += RED_BLOCK)
        s += (double)Ddf<FT>::ld((const typename Ddf<FT>::T*)x, i);
    const double t = block_tree_sum(s, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

static __global__ void __launch_bounds__(RED_BLOCK) k_sum_final(const double* partials, uint32_t nparts,
                                                                double* out) {
    __shared__ double sh[RED_BLOCK];
    double s = 0.0;
    for (uint32_t i = threadIdx.x; i < nparts; i += RED_BLOCK) s += partials[i];
    const double t = block_tree_sum(s, sh);
    if (threadIdx.x == 0) *out = t;
}

// both passes on stream s: nparts blocks of `per` values each (nparts * per >= count)
static inline void launch_sum_two_pass(const void* x, int ft, uint64_t count, uint64_t per, uint32_t nparts,
                                       double* partials, double* out, cudaStream_t s) {
    if (ft == ION_FP32) k_sum_partial<ION_FP32><<<nparts, RED_BLOCK, 0, s>>>(x, count, per, partials);
    else if (ft == ION_FP16S) k_sum_partial<ION_FP16S><<<nparts, RED_BLOCK, 0, s>>>(x, count, per, partials);
    else k_sum_partial<ION_FP16C><<<nparts, RED_BLOCK, 0, s>>>(x, count, per, partials);
    k_sum_final<<<1, RED_BLOCK, 0, s>>>(partials, nparts, out);
}

}  // namespace ion
