// batch_kernels.cu -- many independent domains of uneven size, one launch per
// timestep (no reference counterpart: the reference steps one domain per
// OpenCL queue, src/lbm/mod.rs:250-272).
//
// Two persistent launches advance every domain of a batch by one step:
// k_batch_stream (cooperative) runs
//   A  stream_collide of every cell of every domain   (sc_cell)
//   B  LOD bin sums of every domain                     (lod_bin_warp)
// separated by a grid-wide barrier, and k_batch_field runs
//   C  E/B update of every cell of every domain         (eb_tile)
// (the kernel boundary orders C after B; each kernel has its own register budget).
// Work is handed out in tiles of EB_CPT*blockDim consecutive cells (A), bricks
// or half bricks (C, as in the single-domain E/B kernel) or one warp per bin
// (B); a tile's domain is found by binary search over prefix sums of the
// per-domain tile counts.  Every cell runs exactly the per-cell code of the
// single-domain kernels, so a batched step is bit-identical to stepping the
// domains one by one.  The grid barrier spins with an iteration limit and
// reports a timeout through an error flag instead of hanging.
#include "field_kernels.cuh"
#include "ion_launch.h"
#include "lbm_kernels.cuh"

namespace ion {


__device__ __forceinline__ uint32_t find_domain(const uint32_t* off, uint32_t ndom, uint32_t idx) {
    uint32_t lo = 0, hi = ndom;  // off[lo] <= idx < off[hi]
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= idx) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Generation barrier over all blocks of a co-resident grid.  Returns false
// (block-uniform) when it gave up after `limit` polls.
__device__ __forceinline__ bool grid_barrier(uint32_t* count, uint32_t* gen, uint32_t nblocks, uint32_t limit) {
    __syncthreads();
    int ok = 1;
    if (threadIdx.x == 0) {
        const uint32_t g = *(volatile uint32_t*)gen;
        __threadfence();
        if (atomicAdd(count, 1u) == nblocks - 1u) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            uint32_t i = 0;
            while (*(volatile uint32_t*)gen == g) {
                if (++i > limit) { ok = 0; break; }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    return __syncthreads_and(ok) != 0;
}

// Phase A (+ B with MHD): stream_collide of every cell of every domain, a grid barrier,
// then the LOD bin sums; a cooperative launch of BATCH_SC_THREADS-thread blocks.  It has
// its own register budget (the global-load MHD stencil wants ~140 registers; in one
// kernel with the E/B phase both were held to 128 and spilled).
template <int FT, bool MHD>
__global__ void __launch_bounds__(BATCH_SC_THREADS, MHD ? 3 : 4) k_batch_stream(const BatchDev B, const uint32_t odd_t) {
    __shared__ DevLbm sL;
    __shared__ uint32_t s_dom;
    const bool odd = odd_t != 0u;
    const uint32_t nblocks = gridDim.x;
    for (uint32_t t = blockIdx.x; t < B.total_tiles; t += nblocks) {
        __syncthreads();
        if (threadIdx.x == 0) {
            s_dom = find_domain(B.tile_off, B.ndom, t);
            sL = B.doms[s_dom];
        }
        __syncthreads();
        const uint32_t base = (t - B.tile_off[s_dom]) * blockDim.x * EB_CPT;
        for (uint32_t k = 0; k < EB_CPT; k++) {
            const uint32_t n = base + k * blockDim.x + threadIdx.x;
            if (n < sL.n) {
                if (sL.trt) sc_cell<19, FT, MHD, true>(sL, n, odd);
                else sc_cell<19, FT, MHD, false>(sL, n, odd);
            }
        }
    }
    if constexpr (MHD) {
        if (!grid_barrier(B.bar_count, B.bar_gen, nblocks, B.barrier_limit)) { if (threadIdx.x == 0) atomicExch(B.err, 2u); return; }
        // phase B: LOD bins, one warp per bin
        const uint32_t warps = nblocks * (blockDim.x >> 5);
        for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < B.total_bins; w += warps) {
            const uint32_t d = find_domain(B.bin_off, B.ndom, w);
            const DevLbm& L = B.doms[d];
            if (L.depth > 0u) lod_bin_warp(L, w - B.bin_off[d], threadIdx.x & 31u);
            else if ((threadIdx.x & 31u) < 4u) L.qu_lod[threadIdx.x & 31u] = 0.0f;
        }
    }
}

// Phase C: the E/B update of every brick (or half brick) of every domain, after phase B
// in stream order; blocks walk the bricks grid-stride (launch shape from the autotuner)
template <bool FAST>
__global__ void __launch_bounds__(256, 2) k_batch_field(const BatchDev B) {
    __shared__ __align__(16) EbSmem<FAST> sm;
    __shared__ DevLbm sL;
    __shared__ uint32_t s_dom;
    eb_init(sm);
    uint32_t uses[2] = {0u, 0u};
    const uint32_t parts = 256u / blockDim.x;  // tiles per brick
    for (uint32_t t = blockIdx.x; t < B.total_bricks; t += gridDim.x) {
        __syncthreads();
        if (threadIdx.x == 0) {
            s_dom = find_domain(B.brick_off, B.ndom, t);
            sL = B.doms[s_dom];
        }
        __syncthreads();
        const uint32_t local = t - B.brick_off[s_dom];
        if (!eb_tile<FAST>(sL, local / parts, local % parts, sm, uses)) {
            if (threadIdx.x == 0) atomicExch(B.err, 1u);
            return;
        }
    }
}

static const void* stream_kernel(int ft, bool mhd) {
    if (ft == ION_FP32) return mhd ? (const void*)k_batch_stream<ION_FP32, true> : (const void*)k_batch_stream<ION_FP32, false>;
    if (ft == ION_FP16S) return mhd ? (const void*)k_batch_stream<ION_FP16S, true> : (const void*)k_batch_stream<ION_FP16S, false>;
    return mhd ? (const void*)k_batch_stream<ION_FP16C, true> : (const void*)k_batch_stream<ION_FP16C, false>;
}
static const void* field_kernel(bool fast) { return fast ? (const void*)k_batch_field<true> : (const void*)k_batch_field<false>; }

// blocks per SM of the E/B kernel at `block` threads (the autotuner's range); for
// batches without MHD the stencil kernel's
int batch_max_blocks_per_sm(int ft, bool mhd, bool fast, int block) {
    int n = 0;
    const void* k = mhd ? field_kernel(fast) : stream_kernel(ft, mhd);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, mhd ? block : (int)BATCH_SC_THREADS, 0) != cudaSuccess) return 0;
    return n;
}

// One timestep of a batch: the cooperative stencil (+ bins) kernel at full occupancy,
// then, with MHD, the E/B kernel with the tuned shape (grid x block).
cudaError_t launch_batch_step(const BatchDev& B, int ft, bool mhd, bool fast, uint32_t grid, uint32_t block,
                              uint64_t t, cudaStream_t s) {
    const void* ks = stream_kernel(ft, mhd);
    int per_sm = 0, dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ks, (int)BATCH_SC_THREADS, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint32_t odd = (uint32_t)(t & 1u);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((uint32_t)(per_sm * sms));
    cfg.blockDim = dim3(BATCH_SC_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {(void*)&B, (void*)&odd};
    e = cudaLaunchKernelExC(&cfg, ks, args);
    if (e != cudaSuccess || !mhd) return e;
    cudaLaunchConfig_t cf = {};
    cf.gridDim = dim3(grid);
    cf.blockDim = dim3(block);
    cf.dynamicSmemBytes = 0;
    cf.stream = s;
    void* fargs[] = {(void*)&B};
    return cudaLaunchKernelExC(&cf, field_kernel(fast), fargs);
}

}  // namespace ion
