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

// Phase B (MHD): a grid barrier, then the LOD bins of every domain, one warp per bin
__device__ __forceinline__ void batch_lod_phase(const BatchDev& B) {
    const uint32_t nblocks = gridDim.x;
    if (!grid_barrier(B.bar_count, B.bar_gen, nblocks, B.barrier_limit)) {
        if (threadIdx.x == 0) atomicExch(B.err, 2u);
        return;
    }
    const uint32_t warps = nblocks * (blockDim.x >> 5);
    for (uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < B.total_bins; w += warps) {
        const uint32_t d = find_domain(B.bin_off, B.ndom, w);
        const DevLbm& L = B.doms[d];
        if (L.depth > 0u) lod_bin_warp(L, w - B.bin_off[d], threadIdx.x & 31u);
        else if ((threadIdx.x & 31u) < 4u) L.qu_lod[threadIdx.x & 31u] = 0.0f;
    }
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
    if constexpr (MHD) batch_lod_phase(B);
}

// Phase A (+ B with MHD) over x-rows, when every domain's rows are whole 16-byte streams of
// at most BATCH_ROW_MAX cells: the producer-warp form of k_sc_rows_ws (lbm_kernels.cuh)
// walking the rows of all domains (global row g = blockIdx.x + k gridDim.x, its domain by
// binary search over the prefix sums of ny nz).  The last warp stages each row and writes
// the new DDFs back from the staged rows; the others run sc_cell on the row's cells (one
// per thread).  A row's domain view is copied into the buffer's shared-memory slot when it
// changes.  Per cell it runs sc_cell exactly as the single-domain row kernel does, so the
// results are those of stepping the domains one by one.
template <int FT, bool MHD>
__global__ void __launch_bounds__(BATCH_SC_THREADS, 5) k_batch_stream_rows(const BatchDev B, const uint32_t odd_t) {
    using T = typename Ddf<FT>::T;
    constexpr uint32_t RS = BATCH_ROW_STRIDE;
    constexpr uint32_t RB = ws_row_bytes<FT, MHD, RS>();
    constexpr uint32_t SB = RS * (uint32_t)sizeof(T);  // bytes per stream row
    constexpr uint32_t eb_off = row_streams<FT, MHD>() * SB, fl_off = eb_off + (MHD ? 6u * RS * 4u : 0u);
    extern __shared__ __align__(128) uint8_t rows_smem[];
    __shared__ __align__(8) uint64_t full[2], empty[2];
    __shared__ DevLbm sL[2];                            // the domain of the row in each buffer
    __shared__ uint32_t sdom[2], srow[2], fail_flag, issued;
    volatile uint32_t* fail = &fail_flag;
    const bool odd = odd_t != 0u;
    const uint32_t nct = blockDim.x - 32u, ncw = nct / 32u;  // compute threads and warps
    const uint32_t G = gridDim.x, nrows = B.total_rows;
    const uint32_t limit = B.doms[0].wait_limit;
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1u);
        mbar_init(&full[1], 1u);
        mbar_init(&empty[0], ncw);
        mbar_init(&empty[1], ncw);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fail_flag = 0u;
        issued = 0u;
        sdom[0] = sdom[1] = 0xFFFFFFFFu;
    }
    __syncthreads();
    const uint32_t my_rows = blockIdx.x < nrows ? (nrows - 1u - blockIdx.x) / G + 1u : 0u;
    if (threadIdx.x >= nct) {
        if (threadIdx.x == nct) {
            // row k of this CTA lives in buffer k & 1
            auto write_back = [&](uint32_t k) {
                const uint32_t b = k & 1u;
                const DevLbm& L = sL[b];
                const uint8_t* src = rows_smem + b * RB;
                const uint32_t rb = L.nx * (uint32_t)sizeof(T);
                for_row_streams<FT, MHD>(L, srow[b], odd, [&](uint32_t st, T* g) { bulk_s2g(g, src + st * SB, rb); });
                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            };
            uint32_t k = 0;
            for (; k < my_rows; k++) {
                const uint32_t b = k & 1u, g = blockIdx.x + k * G;
                if (k >= 2) {
                    // row k - 2 computed: copy it back, and wait until the copies have read the buffer
                    if (!mbar_wait_or_fail(&empty[b], ((k - 2) >> 1) & 1u, fail, limit)) break;
                    if (*fail) break;
                    write_back(k - 2u);
                    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                }
                if (*fail) break;
                const uint32_t d = find_domain(B.row_off, B.ndom, g), r = g - B.row_off[d];
                if (sdom[b] != d) {
                    sL[b] = B.doms[d];
                    sdom[b] = d;
                }
                srow[b] = r;
                const DevLbm& L = sL[b];
                const uint32_t nx = L.nx, N = L.n, own = r * nx, rb = nx * (uint32_t)sizeof(T);
                uint8_t* dst = rows_smem + b * RB;
                // (the arrive below releases the view and row index written above)
                mbar_expect_tx(&full[b], row_streams<FT, MHD>() * rb + (MHD ? 6u * nx * 4u : 0u) + ((nx + 15u) & ~15u));
                for_row_streams<FT, MHD>(L, r, odd, [&](uint32_t st, T* gp) { bulk_g2s(dst + st * SB, gp, rb, &full[b]); });
                if constexpr (MHD) {
                    for (uint32_t c = 0; c < 3; c++) {
                        bulk_g2s(dst + eb_off + c * RS * 4u, L.b_dyn + (size_t)c * N + own, nx * 4u, &full[b]);
                        bulk_g2s(dst + eb_off + (3u + c) * RS * 4u, L.e_dyn + (size_t)c * N + own, nx * 4u, &full[b]);
                    }
                }
                bulk_g2s(dst + fl_off, L.flags + own, (nx + 15u) & ~15u, &full[b]);
                issued = k + 1u;
            }
            // the last (up to) two rows, once computed
            if (k == my_rows) {
                for (uint32_t t = my_rows > 2u ? my_rows - 2u : 0u; t < my_rows; t++) {
                    if (!mbar_wait_or_fail(&empty[t & 1u], (t >> 1) & 1u, fail, limit) || *fail) break;
                    write_back(t);
                }
            }
            asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        }
        __syncwarp();
    } else {
        const uint32_t lane = threadIdx.x & 31u;
        for (uint32_t k = 0; k < my_rows; k++) {
            const uint32_t b = k & 1u;
            const bool go = mbar_wait_or_fail(&full[b], (k >> 1) & 1u, fail, limit) && *fail == 0u;
            if (go) {
                const DevLbm& L = sL[b];
                const uint32_t nx = L.nx, r = srow[b];
                uint8_t* buf = rows_smem + b * RB;
                for (uint32_t x = threadIdx.x; x < nx; x += nct) {
                    const RowSrc<T, RS, true> S{buf, nx, x, x + 1u == nx ? 0u : x + 1u, x == 0u ? nx - 1u : x - 1u,
                                                 eb_off, fl_off};
                    if (L.trt) sc_cell<19, FT, MHD, true, false, RowSrc<T, RS, true>, uint32_t>(L, x + r * nx, odd, S);
                    else sc_cell<19, FT, MHD, false, false, RowSrc<T, RS, true>, uint32_t>(L, x + r * nx, odd, S);
                }
                // the new DDFs (generic-proxy writes) become visible to the bulk copies
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            }
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&empty[b])) : "memory");
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && *fail) {
        // copies that may still be in flight: the last two rows the producer staged
        const uint32_t n_issued = issued;
        for (uint32_t k = n_issued > 2u ? n_issued - 2u : 0u; k < n_issued; k++)
            mbar_wait(&full[k & 1u], (k >> 1) & 1u, WAIT_LIMIT);
        atomicExch(B.err, 1u);
    }
    if constexpr (MHD) batch_lod_phase(B);
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

static const void* stream_kernel(int ft, bool mhd, bool rows) {
    if (rows) {
        if (ft == ION_FP32)
            return mhd ? (const void*)k_batch_stream_rows<ION_FP32, true> : (const void*)k_batch_stream_rows<ION_FP32, false>;
        if (ft == ION_FP16S)
            return mhd ? (const void*)k_batch_stream_rows<ION_FP16S, true> : (const void*)k_batch_stream_rows<ION_FP16S, false>;
        return mhd ? (const void*)k_batch_stream_rows<ION_FP16C, true> : (const void*)k_batch_stream_rows<ION_FP16C, false>;
    }
    if (ft == ION_FP32) return mhd ? (const void*)k_batch_stream<ION_FP32, true> : (const void*)k_batch_stream<ION_FP32, false>;
    if (ft == ION_FP16S) return mhd ? (const void*)k_batch_stream<ION_FP16S, true> : (const void*)k_batch_stream<ION_FP16S, false>;
    return mhd ? (const void*)k_batch_stream<ION_FP16C, true> : (const void*)k_batch_stream<ION_FP16C, false>;
}
// dynamic shared memory of the stencil kernel: two row buffers for the row-staged form
static uint32_t stream_smem(int ft, bool mhd, bool rows) {
    if (!rows) return 0u;
    constexpr uint32_t RS = BATCH_ROW_STRIDE;
    if (ft == ION_FP32) return 2u * (mhd ? ws_row_bytes<ION_FP32, true, RS>() : ws_row_bytes<ION_FP32, false, RS>());
    return 2u * (mhd ? ws_row_bytes<ION_FP16S, true, RS>() : ws_row_bytes<ION_FP16S, false, RS>());
}
static const void* field_kernel(bool fast) { return fast ? (const void*)k_batch_field<true> : (const void*)k_batch_field<false>; }

// blocks per SM of the E/B kernel at `block` threads (the autotuner's range); for
// batches without MHD the stencil kernel's
int batch_max_blocks_per_sm(int ft, bool mhd, bool fast, bool rows, int block) {
    int n = 0;
    const void* k = mhd ? field_kernel(fast) : stream_kernel(ft, mhd, rows);
    if (!mhd && rows && cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, mhd ? block : (int)BATCH_SC_THREADS,
                                                      mhd ? 0 : stream_smem(ft, mhd, rows)) != cudaSuccess)
        return 0;
    return n;
}

// One timestep of a batch: the cooperative stencil (+ bins) kernel at full occupancy,
// then, with MHD, the E/B kernel with the tuned shape (grid x block).
cudaError_t launch_batch_step(const BatchDev& B, int ft, bool mhd, bool fast, uint32_t grid, uint32_t block,
                              uint64_t t, cudaStream_t s) {
    const bool rows = B.total_rows > 0u;
    const void* ks = stream_kernel(ft, mhd, rows);
    const uint32_t smem = stream_smem(ft, mhd, rows);
    int per_sm = 0, dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess && rows) e = cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ks, (int)BATCH_SC_THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    const uint32_t odd = (uint32_t)(t & 1u);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((uint32_t)(per_sm * sms));
    cfg.blockDim = dim3(BATCH_SC_THREADS);
    cfg.dynamicSmemBytes = smem;
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
