// ion_launch.h -- host-side launchers of the sm_103a kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ion {

struct DevLbm;

inline unsigned grid_for(uint64_t n, unsigned block) {
    const uint64_t g = (n + block - 1) / block;
    return (unsigned)(g ? g : 1);
}

// voxelize_mesh arguments (IonSolver src/mesh.rs:281-343)
struct VoxArgs {
    const float *p0, *p1, *p2;  // device, [ntri][3]
    uint32_t ntri;
    int direction;
    uint32_t columns;
    float x0, y0, z0, x1, y1, z1;  // bounding box +-2
    uint8_t flag;
    float mx, my, mz;
};

constexpr unsigned RED_BLOCK = 256;

// Cells per thread of the E/B update: each staged source is applied to
// EB_CPT cells held in registers.
constexpr uint32_t EB_CPT = 4;
// The E/B update walks a domain in aligned bricks of EB_BX x EB_BY x EB_CPT
// cells (1024 = 256 threads x EB_CPT); thread t of a 256-thread block holds
// the cells (t % EB_BX, t / EB_BX, 0..EB_CPT-1) of its brick, a 128-thread
// block one half of a brick (sub = 0, 1 in y).  FAST coordinates are taken
// relative to the brick's centre, which depends only on the cell.
constexpr uint32_t EB_BX = 16, EB_BY = 16;
inline uint32_t eb_bricks(uint32_t nx, uint32_t ny, uint32_t nz) {
    return ((nx + EB_BX - 1) / EB_BX) * ((ny + EB_BY - 1) / EB_BY) * ((nz + EB_CPT - 1) / EB_CPT);
}

// device view of a batch of domains (batch_kernels.cu)
struct BatchDev {
    const DevLbm* doms;
    uint32_t ndom;
    const uint32_t* tile_off;  // [ndom+1] prefix sums of ceil(n / (EB_CPT * blockDim)) (stream_collide tiles)
    uint32_t total_tiles;
    const uint32_t* brick_off;  // [ndom+1] prefix sums of bricks x (256 / blockDim) (E/B tiles)
    uint32_t total_bricks;
    const uint32_t* bin_off;   // [ndom+1] prefix sums of n_lod_own
    uint32_t total_bins;
    uint32_t* bar_count;
    uint32_t* bar_gen;
    uint32_t* err;
    uint32_t barrier_limit;  // polls before a grid barrier gives up
    const uint32_t* row_off;   // [ndom+1] prefix sums of ny nz (the row-staged stencil), or null
    uint32_t total_rows;       // 0: the stencil runs in tiles of cells with global loads
};
// threads per block of the batch's stencil kernel (its tiles: BATCH_SC_THREADS * EB_CPT cells;
// row-staged: BATCH_SC_THREADS - 32 compute threads, so rows of up to BATCH_ROW_MAX cells,
// staged at a row stride of BATCH_ROW_STRIDE elements: 96 x 4 bytes keeps every stream
// 16-byte aligned, and the smaller buffers fit five CTAs per SM in FP32 MHD)
constexpr uint32_t BATCH_SC_THREADS = 128;
constexpr uint32_t BATCH_ROW_MAX = BATCH_SC_THREADS - 32, BATCH_ROW_STRIDE = BATCH_ROW_MAX;
static_assert(BATCH_ROW_STRIDE % 16 == 0, "row streams of 16-byte multiples in shared memory");
int batch_max_blocks_per_sm(int ft, bool mhd, bool fast, bool rows, int block);
cudaError_t launch_batch_step(const BatchDev& B, int ft, bool mhd, bool fast, uint32_t grid, uint32_t block,
                              uint64_t t, cudaStream_t s);

// per velocity set (lbm_q19.cu, lbm_q15.cu, lbm_q9.cu)
#define ION_DECLARE_LBM_DISPATCH(NAME)                                                                    \
    void NAME##_stream_collide(const DevLbm& L, int ft, int mode, bool trt, uint64_t t, uint32_t* err,       \
                               cudaStream_t s);                                                            \
    void NAME##_initialize(const DevLbm& L, int ft, int mode, cudaStream_t s);                            \
    void NAME##_update_fields(const DevLbm& L, int ft, uint64_t t, cudaStream_t s);
ION_DECLARE_LBM_DISPATCH(q19)
ION_DECLARE_LBM_DISPATCH(q15)
ION_DECLARE_LBM_DISPATCH(q9)

void launch_lod_bins(const DevLbm& L, cudaStream_t s);
void launch_update_e_b(const DevLbm& L, bool fast, uint32_t* err, cudaStream_t s);
void launch_div_check(uint64_t samples, uint64_t seed, unsigned long long* bad, float* first_bad, cudaStream_t s);
void launch_update_e_b_gated(const DevLbm& L, uint32_t* err, const uint32_t* gate, cudaStream_t s);
void launch_voxelize(const DevLbm& L, const VoxArgs& A, cudaStream_t s);
void launch_compact(const DevLbm& L, uint8_t mask, uint32_t* tiles, uint32_t* list, uint32_t* total, cudaStream_t s);
void launch_psi_static_b(const DevLbm& L, const uint32_t* mags, const uint32_t* count, cudaStream_t s);
void launch_static_e(const DevLbm& L, const uint32_t* list, const uint32_t* count, float* E, cudaStream_t s);
void launch_sum_f64(const void* x, int ft, uint64_t count, double* partials, uint32_t nparts, double* out,
                    cudaStream_t s);
void launch_fma_probe(float* out, int blocks, int iters, cudaStream_t s);
void launch_codec(int ft, const float* in, uint16_t* enc, float* dec, const uint16_t* raw, float* raw_dec, uint64_t n,
                  cudaStream_t s);

}  // namespace ion

namespace ion {
// error reporting and launch accounting of the C ABI (ion_api.cu)
int api_fail(int code, const char* message);
void api_count_launches(uint64_t n);
}  // namespace ion
