// batch_kernels.cu -- many independent domains of uneven size, one launch per
// timestep (no reference counterpart: the reference steps one domain per
// OpenCL queue, src/lbm/mod.rs:250-272).
//
// One persistent, cooperatively launched kernel advances every domain of a
// batch by one step in three phases separated by grid-wide barriers:
//   A  stream_collide of every cell of every domain   (sc_cell)
//   B  LOD bin sums of every domain                     (lod_bin_warp)
//   C  E/B update of every cell of every domain         (eb_tile)
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

// At most 128 registers (two 256-thread or four 128-thread blocks per SM): the three
// phases fit with small spills, and the E/B phase needs the warps (8 -> 16 per SM took a
// 96-domain step from 91.5 to 79.2 ms)
template <int FT, bool MHD, bool FAST>
__global__ void __launch_bounds__(256, 2) k_batch_step(const BatchDev B, const uint32_t odd_t) {
    __shared__ __align__(16) EbSmem<FAST> sm;
    __shared__ DevLbm sL;
    __shared__ uint32_t s_dom;
    const bool odd = odd_t != 0u;
    const uint32_t nblocks = gridDim.x;

    // phase A: stream_collide
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
        if (!grid_barrier(B.bar_count, B.bar_gen, nblocks, B.barrier_limit)) { if (threadIdx.x == 0) atomicExch(B.err, 2u); return; }
        // phase C: E/B update
        eb_init(sm);
        uint32_t uses[2] = {0u, 0u};
        const uint32_t parts = 256u / blockDim.x;  // tiles per brick
        for (uint32_t t = blockIdx.x; t < B.total_bricks; t += nblocks) {
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
}

#define ION_BATCH_CASE(FTV, MHDV, FASTV)                                                   \
    if (ft == FTV && mhd == MHDV && fast == FASTV) {                                       \
        kern = (const void*)k_batch_step<FTV, MHDV, FASTV>;                                \
    }

static const void* batch_kernel(int ft, bool mhd, bool fast) {
    const void* kern = nullptr;
    ION_BATCH_CASE(ION_FP32, false, false)
    ION_BATCH_CASE(ION_FP16S, false, false)
    ION_BATCH_CASE(ION_FP16C, false, false)
    ION_BATCH_CASE(ION_FP32, true, false)
    ION_BATCH_CASE(ION_FP16S, true, false)
    ION_BATCH_CASE(ION_FP16C, true, false)
    ION_BATCH_CASE(ION_FP32, true, true)
    ION_BATCH_CASE(ION_FP16S, true, true)
    ION_BATCH_CASE(ION_FP16C, true, true)
    return kern;
}

int batch_max_blocks_per_sm(int ft, bool mhd, bool fast, int block) {
    int n = 0;
    const void* k = batch_kernel(ft, mhd, fast);
    if (!k || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, block, 0) != cudaSuccess) return 0;
    return n;
}

cudaError_t launch_batch_step(const BatchDev& B, int ft, bool mhd, bool fast, uint32_t grid, uint32_t block,
                              uint64_t t, cudaStream_t s) {
    const void* k = batch_kernel(ft, mhd, fast);
    if (!k) return cudaErrorInvalidValue;
    const uint32_t odd = (uint32_t)(t & 1u);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {(void*)&B, (void*)&odd};
    return cudaLaunchKernelExC(&cfg, k, args);
}

}  // namespace ion
