// noalloc.cu -- FP64 sum of stored DDFs that allocates no device memory.
//
// Some callers cannot call cudaMalloc/cudaFree at the point where they need
// this sum: a host program whose device memory is already fully reserved by
// its own pool allocator, or a time-stepping loop that must not pay the
// implicit device synchronisation cudaFree performs.  ion_ddf_sum_f64_noalloc
// gives them the same reduction as the one behind ion_lbm_mass_charge, with
// its scratch (one double per block) in a fixed array in device memory that
// exists, on every GPU that loads this library, until the process exits.
//
// Rules of use:
//   - the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture on that device;
//   - every call on a device shares the one array: two calls whose kernels
//     overlap on the GPU (different streams, no ordering between them) race
//     and give wrong sums; order them on one stream or synchronise;
//   - each call overwrites exactly the partials it later reads, so nothing
//     carries over from the previous call;
//   - at most ION_NOALLOC_MAX_VALUES values per call (ION_E_INVALID beyond).
#include <mutex>

#include "ion_device.cuh"
#include "ion_launch.h"

namespace ion {

// 4096 partial sums (32 KiB); each covers NOALLOC_PER_PART values.
constexpr uint32_t NOALLOC_PARTS = 4096;
constexpr uint64_t NOALLOC_PER_PART = 1ull << 16;
static __device__ __align__(256) double g_noalloc_partials[NOALLOC_PARTS];

template <int FT>
__global__ void __launch_bounds__(RED_BLOCK) k_noalloc_partial(const void* x, uint64_t count, double* partials) {
    __shared__ double sh[RED_BLOCK];
    const uint64_t b = (uint64_t)blockIdx.x * NOALLOC_PER_PART;
    const uint64_t e = min(b + NOALLOC_PER_PART, count);
    double s = 0.0;
    for (uint64_t i = b + threadIdx.x; i < e; i += RED_BLOCK)
        s += (double)Ddf<FT>::ld((const typename Ddf<FT>::T*)x, i);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = RED_BLOCK / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(RED_BLOCK) k_noalloc_final(const double* partials, uint32_t nparts, double* out) {
    __shared__ double sh[RED_BLOCK];
    double s = 0.0;
    for (uint32_t i = threadIdx.x; i < nparts; i += RED_BLOCK) s += partials[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = RED_BLOCK / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// device address of g_noalloc_partials, looked up once per device
static double* scratch_for_current_device(cudaError_t* err) {
    constexpr int MAX_DEV = 64;
    static std::mutex mu;
    static double* addr[MAX_DEV] = {};
    int dev = 0;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess) return nullptr;
    if (dev < 0 || dev >= MAX_DEV) { *err = cudaErrorInvalidDevice; return nullptr; }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        *err = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (*err != cudaSuccess) return nullptr;
        addr[dev] = (double*)p;
    }
    return addr[dev];
}

}  // namespace ion

extern "C" int ion_ddf_sum_f64_noalloc(const void* d_values, int float_type, uint64_t count, double* d_sum,
                                       void* stream) {
    using namespace ion;
    if (!d_values || !d_sum) return api_fail(ION_E_INVALID, "null device pointer");
    if (float_type < ION_FP16S || float_type > ION_FP32) return api_fail(ION_E_INVALID, "unknown float_type");
    if (count == 0) return api_fail(ION_E_INVALID, "count is 0");
    if (count > (uint64_t)NOALLOC_PARTS * NOALLOC_PER_PART)
        return api_fail(ION_E_INVALID, "count exceeds ION_NOALLOC_MAX_VALUES (268435456 values per call)");
    cudaError_t e = cudaSuccess;
    double* partials = scratch_for_current_device(&e);
    if (!partials) return api_fail(ION_E_CUDA, cudaGetErrorString(e));
    const uint32_t nparts = (uint32_t)((count + NOALLOC_PER_PART - 1) / NOALLOC_PER_PART);
    cudaStream_t s = (cudaStream_t)stream;
    if (float_type == ION_FP32) k_noalloc_partial<ION_FP32><<<nparts, RED_BLOCK, 0, s>>>(d_values, count, partials);
    else if (float_type == ION_FP16S) k_noalloc_partial<ION_FP16S><<<nparts, RED_BLOCK, 0, s>>>(d_values, count, partials);
    else k_noalloc_partial<ION_FP16C><<<nparts, RED_BLOCK, 0, s>>>(d_values, count, partials);
    k_noalloc_final<<<1, RED_BLOCK, 0, s>>>(partials, nparts, d_sum);
    api_count_launches(2);
    e = cudaGetLastError();
    if (e != cudaSuccess) return api_fail(ION_E_CUDA, cudaGetErrorString(e));
    return ION_OK;
}
