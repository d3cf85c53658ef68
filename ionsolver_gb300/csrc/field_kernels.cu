// field_kernels.cu -- launchers of the LOD-bin and E/B kernels (field_kernels.cuh).
#include "field_kernels.cuh"

namespace ion {

void launch_lod_bins(const DevLbm& L, cudaStream_t s) {
    k_lod_bins<<<L.n_lod_own, LB_THREADS, 0, s>>>(L);
}

void launch_update_e_b_gated(const DevLbm& L, uint32_t* err, const uint32_t* gate, cudaStream_t s) {
    k_update_e_b_gated<<<eb_bricks(L.nx, L.ny, L.nz), 256, 0, s>>>(L, err, gate);
}

void launch_update_e_b(const DevLbm& L, bool fast, uint32_t* err, cudaStream_t s) {
    const unsigned g = eb_bricks(L.nx, L.ny, L.nz);
    if (fast) k_update_e_b_fast<<<g, 256, 0, s>>>(L, err);
    else k_update_e_b_exact<<<g, 256, 0, s>>>(L, err);
}

}  // namespace ion
