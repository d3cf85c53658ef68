// surrogate.h -- the learned far field of the E/B update (surrogate.cu).
#pragma once
#include <cstdint>
#include <random>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "ion_device.cuh"

namespace ion {

// the tcgen05 convolution against the mma.sync one (self-test, see surrogate.cu)
int conv_tc_selftest(int nd, int cin, int cout, int dil, uint64_t seed, float* max_rel, cudaStream_t s);

class Surrogate {
public:
    static constexpr int RNEAR = 1;           // bins within this Chebyshev distance are summed exactly
    static constexpr int NEAR_SIDE = 2 * RNEAR + 1, NEAR_CAND = NEAR_SIDE * NEAR_SIDE * NEAR_SIDE;
    static constexpr int NODES = 27;          // 3 x 3 x 3 interpolation nodes per block
    static constexpr int OUT_CH = NODES * 6;  // (Ex,Ey,Ez,Bx,By,Bz) per node
    static constexpr int OUT_PAD = 168;       // head channels: OUT_CH rounded up to 8 (the rest are zero)
    static constexpr int MAX_BLOCK = 32;      // largest LOD block edge (cells) the per-cell kernel tabulates
    ~Surrogate();
    int init(int nd, float bsx, float bsy, float bsz, int first_src);
    // generates `nsamples` snapshots (random charge/current per bin, exact far-field
    // targets), trains with Adam, returns the held-out relative L2 error of the BF16 path
    int train(int nsamples, int epochs, int batch, float lr, uint64_t seed, cudaStream_t s, float* rel_err);
    int save(const char* path) const;
    int load(const char* path, cudaStream_t s);
    // one step: source scales, network input, BF16 inference, per-cell field,
    // sampled exact check and the fallback decision (device flag)
    void step(const DevLbm& L, cudaStream_t s, uint32_t salt);
    uint32_t launches_per_step() const;
    bool ready() const { return ready_; }
    const uint32_t* fallback_flag() const { return flag_; }
    // tolerance and sample size of the check; restarts the statistics (and so the sample sequence)
    void configure(float tol, uint32_t cells, cudaStream_t s) {
        tol_ = tol;
        check_cells_ = cells;
        cudaMemsetAsync(counters_, 0, 3 * sizeof(unsigned long long), s);
    }
    float tol() const { return tol_; }
    uint32_t check_cells() const { return check_cells_; }
    // counters: [0] checks, [1] fallbacks, [2] checks that saw a non-finite exact field; last: relative errors
    void stats_device(unsigned long long** counters, float** last) { *counters = counters_; *last = last_; }
    float rel32() const { return rel32_; }
    float rel16() const { return rel16_; }
    const std::vector<float>& loss_history() const { return loss_; }
    void infer_bf16(const float* X, cudaStream_t s);
    size_t weight_count() const { return nw_; }
    int get_weights(float* host) const;
    int set_weights(const float* host, cudaStream_t s);
    // loss and weight gradient of one batch (host arrays; targets in the network's output scale)
    int grad(const float* hX, const float* hT, int B, float* loss, float* hgrad, cudaStream_t s);
    // exact far-field targets (unscaled) of B source snapshots (host arrays)
    int targets(const float* hX, float* hT, int B, cudaStream_t s);
    float out_scale_e() const { return yE_; }
    float out_scale_b() const { return yB_; }
    // FP32 (bf16=false) or BF16 tensor-core (bf16=true) forward of one sample (host arrays)
    int forward(const float* hX, float* hY, bool bf16, cudaStream_t s);

private:
    int alloc(void** p, size_t bytes);
    int reset_weights(uint64_t seed);
    void forward_fp32(const float* X, int B, std::vector<float*>& acts, float* Y, cudaStream_t s);
    void backward_fp32(const float* X, int B, std::vector<float*>& acts, const float* gY, std::vector<float*>& g,
                       cudaStream_t s);
    void pack_bf16(cudaStream_t s);
    void make_snapshot(std::mt19937_64& gen, float* x) const;
    void k_pack_input_dev(const DevLbm& L, cudaStream_t s);

    int nd_ = 0, V_ = 0, first_ = 0;
    float bs_[3] = {1, 1, 1};
    size_t woff_[10] = {}, wkoff_[10] = {};  // FP32 weights [co][ci][27]; packed BF16 [co][27][ci (>= 16)]
    size_t nw_ = 0, nwk_ = 0;
    float *w_ = nullptr, *gw_ = nullptr, *m_ = nullptr, *v_ = nullptr, *wt_ = nullptr;
    __nv_bfloat16* wk_ = nullptr;
    float *scales_ = nullptr, *last_ = nullptr, *xin_ = nullptr, *yout_ = nullptr, *ha_ = nullptr;
    float* gunit_ = nullptr;  // far field of unit sources in every source bin, [OUT_PAD][V]
    __nv_bfloat16 *ab_ = nullptr, *bb_ = nullptr, *xb_ = nullptr;
    uint32_t *stats_ = nullptr, *flag_ = nullptr;
    unsigned long long* counters_ = nullptr;
    float yE_ = 1.0f, yB_ = 1.0f;
    float tol_ = 1e-2f;
    uint32_t check_cells_ = 1024;
    float rel32_ = -1.0f, rel16_ = -1.0f;
    bool ready_ = false;
    uint64_t seed_ = 12345;
    std::vector<float> loss_;
    std::vector<void*> allocs_;
};

}  // namespace ion
