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
//   - the looked-up address is kept for the life of the process: after
//     cudaDeviceReset (or any other teardown of the device's primary context)
//     it is stale, and calls on that device are not supported any more;
//   - at most ION_NOALLOC_MAX_VALUES values per call (ION_E_INVALID beyond).
#include <mutex>

#include "ion_device.cuh"
#include "ion_launch.h"
#include "reduce_f64.cuh"

namespace ion {

// 4096 partial sums (32 KiB); each covers NOALLOC_PER_PART values.
constexpr uint32_t NOALLOC_PARTS = 4096;
constexpr uint64_t NOALLOC_PER_PART = 1ull << 16;
static __device__ __align__(256) double g_noalloc_partials[NOALLOC_PARTS];

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
    // the shared two-pass sum (reduce_f64.cuh) with blocks of NOALLOC_PER_PART values
    launch_sum_two_pass(d_values, float_type, count, NOALLOC_PER_PART, nparts, partials, d_sum, (cudaStream_t)stream);
    api_count_launches(2);
    e = cudaGetLastError();
    if (e != cudaSuccess) return api_fail(ION_E_CUDA, cudaGetErrorString(e));
    return ION_OK;
}
