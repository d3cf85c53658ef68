// surrogate.cu -- learned far field for the E/B update (no reference
// counterpart; it stands in for the far part of update_e_b_dynamic,
// IonSolver src/kernels/sim_kernels.cl:940-955).
//
// Split of the reference's sum over the depth-D LOD bins of one cell:
//   near : bins within Chebyshev distance RNEAR (= 1) of the cell's own bin
//          (own bin excluded, as the reference excludes it) -- summed exactly
//          per cell (<= 124 terms instead of ~4095);
//   far  : all other bins in range -- smooth over one block, so it is taken
//          at 3 x 3 x 3 nodes of the cell's block (corners, edge and face
//          midpoints, centre) and interpolated with triquadratic Lagrange
//          weights.  The 27 x 6 node values of every block come from a
//          bias-free (linear) 3-D convolutional network on the LOD grid:
//          4 input channels (q, q vx, q vy, q vz per bin), 32 hidden
//          channels, 4 residual blocks of two 3^3 convolutions (dilations
//          (1,2) (2,4) (4,8) (1,1)), 168 output channels (162 used).  The
//          target map is linear in the sources, so the network is kept
//          linear: scaling the inputs scales the outputs exactly.
// Training runs on the GPU with the kernels below (FP32 forward, backward
// of data and weights, Adam); inference runs in BF16 on the tensor cores
// (mma.sync m16n8k16, FP32 accumulation).  Each step a sampled-cell check
// compares the written field with the exact sum on a few cells; above the
// tolerance the exact kernel recomputes the whole field.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include <cuda_bf16.h>

#include "field_kernels.cuh"
#include "tcgen05.cuh"
#include "ion_launch.h"
#include "surrogate.h"

namespace ion {

// ---------------------------------------------------------------------------
// geometry helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ int tap_off(int k, int a) { return (a == 0 ? k % 3 : a == 1 ? (k / 3) % 3 : k / 9) - 1; }

// ---------------------------------------------------------------------------
// exact far-field targets at the 27 nodes of every block
//   src [4][V]: (q, qvx, qvy, qvz) per bin (bins below first_src are 0)
//   out [OUT_PAD][V]: channel = node * 6 + component (Ex,Ey,Ez,Bx,By,Bz),
//   node = ix + 3 (iy + 3 iz) at cell offset (i / 2) (bs - 1) on each axis;
//   channels >= OUT_CH are left as they are (zero).
// FP32 with IEEE sqrt and divide; the sum runs over bins in ascending order.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_far_targets(const float* src, int nd, float bs_x, float bs_y, float bs_z,
                                                     int rnear, float* out, int nsamples) {
    constexpr int NODES = Surrogate::NODES;
    const int V = nd * nd * nd;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)V * NODES * nsamples) return;
    const int s = (int)(gid / (V * NODES));
    const int r = (int)(gid % (V * NODES));
    const int v = r / NODES, node = r % NODES;
    const int bx = v % nd, by = (v / nd) % nd, bz = v / (nd * nd);
    const float tx = 0.5f * (float)(node % 3), ty = 0.5f * (float)((node / 3) % 3), tz = 0.5f * (float)(node / 9);
    const float px = bx * bs_x + tx * (bs_x - 1.0f);
    const float py = by * bs_y + ty * (bs_y - 1.0f);
    const float pz = bz * bs_z + tz * (bs_z - 1.0f);
    const float* S = src + (size_t)s * 4 * V;
    float e[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    for (int d = 0; d < V; d++) {
        const int dx = d % nd, dy = (d / nd) % nd, dz = d / (nd * nd);
        const int cheb = max(abs(dx - bx), max(abs(dy - by), abs(dz - bz)));
        if (cheb <= rnear) continue;
        const float q = S[d];
        const float qx = S[V + d], qy = S[2 * V + d], qz = S[3 * V + d];
        const float Rx = px - (dx * bs_x + 0.5f * bs_x), Ry = py - (dy * bs_y + 0.5f * bs_y);
        const float Rz = pz - (dz * bs_z + 0.5f * bs_z);
        const float r2 = Rx * Rx + Ry * Ry + Rz * Rz;
        const float inv3 = 1.0f / (r2 * sqrtf(r2));
        e[0] += q * Rx * inv3; e[1] += q * Ry * inv3; e[2] += q * Rz * inv3;
        b[0] += (qy * Rz - qz * Ry) * inv3; b[1] += (qz * Rx - qx * Rz) * inv3; b[2] += (qx * Ry - qy * Rx) * inv3;
    }
    float* O = out + (size_t)s * Surrogate::OUT_PAD * V;
    for (int c = 0; c < 3; c++) {
        O[(node * 6 + c) * V + v] = e[c];
        O[(node * 6 + 3 + c) * V + v] = b[c];
    }
}

// divides the E channels by yE and the B channels by yB (network output scale)
__global__ void k_scale_targets(float* T, int V, size_t total, float inv_e, float inv_b) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int ch = (int)((i / V) % Surrogate::OUT_PAD);
    T[i] *= (ch % 6 < 3) ? inv_e : inv_b;
}

// ---------------------------------------------------------------------------
// FP32 training kernels
// ---------------------------------------------------------------------------
constexpr int COG = 8;  // output channels per thread

// out[b][co][v] = (res ? res[b][co][v] : 0) + sum_ci sum_k w[co][ci][k] in[b][ci][v + dil*off_k]
// (weights staged through shared memory CI_CHUNK input channels at a time)
constexpr int CI_CHUNK = 32;
__global__ void __launch_bounds__(128) k_conv_fwd(const float* in, const float* w, const float* res, float* out, int Cin,
                                                  int Cout, int dil, int nd, int B) {
    __shared__ float sw[COG * CI_CHUNK * 27];
    const int V = nd * nd * nd;
    const int co0 = blockIdx.y * COG;
    const int ncog = min(COG, Cout - co0);
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = gid < (long long)B * V;
    const int b = live ? (int)(gid / V) : 0, v = live ? (int)(gid % V) : 0;
    const int x = v % nd, y = (v / nd) % nd, z = v / (nd * nd);
    float acc[COG];
#pragma unroll
    for (int j = 0; j < COG; j++) acc[j] = 0.0f;
    const float* I = in + (size_t)b * Cin * V;
    for (int ci0 = 0; ci0 < Cin; ci0 += CI_CHUNK) {
        const int nci = min(CI_CHUNK, Cin - ci0);
        __syncthreads();
        for (int i = threadIdx.x; i < ncog * nci * 27; i += blockDim.x) {
            const int j = i / (nci * 27), r = i % (nci * 27);
            sw[(j * CI_CHUNK + r / 27) * 27 + r % 27] = w[((size_t)(co0 + j) * Cin + ci0 + r / 27) * 27 + r % 27];
        }
        __syncthreads();
        if (!live) continue;
        for (int k = 0; k < 27; k++) {
            const int xx = x + dil * tap_off(k, 0), yy = y + dil * tap_off(k, 1), zz = z + dil * tap_off(k, 2);
            if (xx < 0 || yy < 0 || zz < 0 || xx >= nd || yy >= nd || zz >= nd) continue;
            const int nv = xx + (yy + zz * nd) * nd;
            for (int ci = 0; ci < nci; ci++) {
                const float a = I[(size_t)(ci0 + ci) * V + nv];
#pragma unroll
                for (int j = 0; j < COG; j++) acc[j] = fmaf(sw[(j * CI_CHUNK + ci) * 27 + k], a, acc[j]);
            }
        }
    }
    if (!live) return;
    for (int j = 0; j < ncog; j++) {
        const size_t o = ((size_t)b * Cout + co0 + j) * V + v;
        out[o] = (res ? res[o] : 0.0f) + acc[j];
    }
}

// wt[ci][co][k] = w[co][ci][26-k]: the data gradient is the forward conv with these weights
__global__ void k_transpose_flip(const float* w, float* wt, int Cin, int Cout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Cin * Cout * 27) return;
    const int k = i % 27, co = (i / 27) % Cout, ci = i / (27 * Cout);
    wt[i] = w[((size_t)co * Cin + ci) * 27 + (26 - k)];
}

// gw[co][ci][k] = sum_b sum_v gout[b][co][v] in[b][ci][v + dil*off_k]
__global__ void __launch_bounds__(256) k_conv_wgrad(const float* in, const float* gout, float* gw, int Cin, int Cout,
                                                    int dil, int nd, int B) {
    __shared__ float red[256];
    const int V = nd * nd * nd;
    const int co = blockIdx.x / Cin, ci = blockIdx.x % Cin;
    float acc[27];
#pragma unroll
    for (int k = 0; k < 27; k++) acc[k] = 0.0f;
    for (int i = threadIdx.x; i < B * V; i += blockDim.x) {
        const int b = i / V, v = i % V;
        const float g = gout[((size_t)b * Cout + co) * V + v];
        const int x = v % nd, y = (v / nd) % nd, z = v / (nd * nd);
        const float* I = in + ((size_t)b * Cin + ci) * V;
#pragma unroll
        for (int k = 0; k < 27; k++) {
            const int xx = x + dil * tap_off(k, 0), yy = y + dil * tap_off(k, 1), zz = z + dil * tap_off(k, 2);
            if (xx >= 0 && yy >= 0 && zz >= 0 && xx < nd && yy < nd && zz < nd)
                acc[k] = fmaf(g, I[xx + (yy + zz * nd) * nd], acc[k]);
        }
    }
    for (int k = 0; k < 27; k++) {
        red[threadIdx.x] = acc[k];
        __syncthreads();
        for (int off = blockDim.x / 2; off > 0; off >>= 1) {
            if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
            __syncthreads();
        }
        if (threadIdx.x == 0) gw[((size_t)co * Cin + ci) * 27 + k] = red[0];
        __syncthreads();
    }
}

// squared error and its gradient: g = 2 (y - t) / count
__global__ void k_mse(const float* y, const float* t, float* g, float* loss, size_t count) {
    __shared__ float red[256];
    float s = 0.0f;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const float d = y[i] - t[i];
        g[i] = 2.0f * d / (float)count;
        s += d * d;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, red[0]);
}

// Adam (Kingma & Ba 2015) with bias correction
__global__ void k_adam(float* w, const float* g, float* m, float* v, size_t n, float lr, float b1, float b2, float eps,
                       float c1, float c2) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ---------------------------------------------------------------------------
// BF16 tensor-core inference: implicit GEMM per layer, M = voxels, N = Cout,
// K = 27 taps x CIN channels (k = tap * CIN + ci), mma.sync.m16n8k16 (BF16 in,
// FP32 accumulate).  Activations are voxel-major, act [V][CIN] bf16, so the
// two K-neighbours of an A fragment register are one 32-bit load; weights are
// packed wkT [Cout][K] bf16 for the same reason on B.  The 4 input channels
// of the first layer are padded to 16.
//   out fp32 [Cout][V] (+ res), outb bf16 [V][Cout] copy for the next layer
// One warp computes 16 voxels x NTW n-tiles of 8 channels; blockIdx.y picks
// the group of n-tiles.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t ld_b32(const __nv_bfloat16* p) { return *(const uint32_t*)p; }

template <int CIN, int NTW>
__global__ void __launch_bounds__(128) k_conv_bf16(const __nv_bfloat16* act, const __nv_bfloat16* wkT, const float* res,
                                                   float* out, __nv_bfloat16* outb, int Cout, int dil, int nd) {
    static_assert(CIN % 16 == 0, "K steps of 16 stay within one tap");
    constexpr int K = 27 * CIN;
    const int V = nd * nd * nd;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, tg = lane & 3;
    const int v0 = warp * 16;
    if (v0 >= V) return;
    const int nt0 = blockIdx.y * NTW;
    float acc[NTW][4];
#pragma unroll
    for (int t = 0; t < NTW; t++) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.0f;
    // voxel rows owned by this thread in the A fragment: v0 + g and v0 + g + 8
    const int va = v0 + g, vb = v0 + g + 8;
    const int xa = va % nd, ya = (va / nd) % nd, za = va / (nd * nd);
    const int xb = vb % nd, yb = (vb / nd) % nd, zb = vb / (nd * nd);
    const __nv_bfloat16* wrow[NTW];
#pragma unroll
    for (int t = 0; t < NTW; t++) wrow[t] = wkT + (size_t)((nt0 + t) * 8 + g) * K + tg * 2;
    for (int tap = 0; tap < 27; tap++) {
        const int ox = dil * tap_off(tap, 0), oy = dil * tap_off(tap, 1), oz = dil * tap_off(tap, 2);
        const int ax = xa + ox, ay = ya + oy, az = za + oz, bx = xb + ox, by = yb + oy, bz = zb + oz;
        const bool ina = ax >= 0 && ay >= 0 && az >= 0 && ax < nd && ay < nd && az < nd;
        const bool inb = bx >= 0 && by >= 0 && bz >= 0 && bx < nd && by < nd && bz < nd;
        const __nv_bfloat16* pa = act + (size_t)(ina ? ax + (ay + az * nd) * nd : 0) * CIN + tg * 2;
        const __nv_bfloat16* pb = act + (size_t)(inb ? bx + (by + bz * nd) * nd : 0) * CIN + tg * 2;
#pragma unroll
        for (int c0 = 0; c0 < CIN; c0 += 16) {
            // a0:(g, k lo) a1:(g+8, k lo) a2:(g, k hi) a3:(g+8, k hi)
            const uint32_t a0 = ina ? ld_b32(pa + c0) : 0u, a1 = inb ? ld_b32(pb + c0) : 0u;
            const uint32_t a2 = ina ? ld_b32(pa + c0 + 8) : 0u, a3 = inb ? ld_b32(pb + c0 + 8) : 0u;
            const int k0 = tap * CIN + c0;
#pragma unroll
            for (int t = 0; t < NTW; t++) {
                const uint32_t b0 = ld_b32(wrow[t] + k0), b1 = ld_b32(wrow[t] + k0 + 8);
                asm volatile(
                    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                    "{%0,%1,%2,%3};\n"
                    : "+f"(acc[t][0]), "+f"(acc[t][1]), "+f"(acc[t][2]), "+f"(acc[t][3])
                    : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
            }
        }
    }
    // C fragment: (g, n = t*8 + tg*2 + {0,1}) and (g+8, same n)
#pragma unroll
    for (int t = 0; t < NTW; t++) {
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int v = (e < 2) ? va : vb;
            const int n = (nt0 + t) * 8 + tg * 2 + (e & 1);
            const size_t o = (size_t)n * V + v;
            const float val = acc[t][e] + (res ? res[o] : 0.0f);
            out[o] = val;
            if (outb) outb[(size_t)v * Cout + n] = __float2bfloat16(val);
        }
    }
}

// ---------------------------------------------------------------------------
// The same convolution on the 5th-generation tensor cores (tcgen05): one CTA
// of 4 warps per 128 voxels (M = 128), N = output channels padded to a
// multiple of 16 (32 or 176), K walked one tap (CIN channels) at a time.  Per
// tap the CTA gathers the 128 x CIN activation tile and the N x CIN weight
// tile into shared memory in the canonical K-major layout without swizzle
// (8-row x 16-byte core matrices; LBO = 128 B between core matrices along K,
// SBO = CIN/8 x 128 B between 8-row groups), one elected thread issues
// tcgen05.mma.kind::f16 (BF16 x BF16 -> FP32) into a TMEM accumulator of
// 128 lanes x N columns and commits to the tile buffer's mbarrier; the two
// tile buffers alternate, so the gather of tap t+1 overlaps the MMAs of tap
// t.  The epilogue reads the accumulator with tcgen05.ld (warp w owns TMEM
// lanes 32w..32w+31 = voxels), adds the residual and writes FP32 and BF16.
// Waits are bounded; a timeout sets *err and the CTA still frees its TMEM.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async16(void* dst, const void* src, uint32_t bytes) {  // bytes 0: zero fill
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(tc::saddr(dst)), "l"(src), "r"(bytes)
                 : "memory");
}

// 3-D convolution (27 taps, dilation dil, zero padding) as an implicit GEMM on
// the 5th-generation tensor cores: D[voxel][n] = sum over (tap, ci) of
// act[neighbour(voxel, tap)][ci] * wkT[n][tap][ci].  One CTA per 128 voxels
// (the MMA's M) and NP output channels (blockIdx.y picks the chunk); the K loop
// walks the taps, CIN channels each.  Operands are gathered with cp.async into an
// S-stage ring of shared-memory tiles in the no-swizzle K-major core-matrix
// layout (8 rows x 16 bytes per core matrix; LBO 128 bytes between the K
// neighbours, SBO between 8-row groups), so S - 1 taps of loads are in flight
// while the MMAs of the current tap run; one elected thread issues the MMAs
// (accumulator in TMEM) and commits each tap to the mbarrier of its stage, which
// frees the stage for refilling.  The epilogue reads TMEM with tcgen05.ld (warp w:
// lanes 32w..32w+31 = its voxels) and writes out[n][v] = D + res[n][v] (FP32,
// channel-major) and outb[v][n] (BF16, voxel-major: the next layer's input).
// Every mbarrier wait is bounded; a wait that gives up raises *err, waits (bounded)
// for the MMAs already issued, frees TMEM and skips the epilogue.
template <int CIN, int NP, int S>
__global__ void __launch_bounds__(128, 1) k_conv_tc(const __nv_bfloat16* act, const __nv_bfloat16* wkT, const float* res,
                                                   float* out, __nv_bfloat16* outb, int Cout, int dil, int nd,
                                                   uint32_t* err) {
    static_assert(CIN % 16 == 0 && NP % 16 == 0 && NP >= 16 && NP <= 256 && S >= 2, "tcgen05 shape");
    constexpr int K = 27 * CIN;
    constexpr uint32_t KCOL = CIN / 8;             // core-matrix columns per tap
    constexpr uint32_t SBO = KCOL * 128u;          // bytes between 8-row groups
    constexpr uint32_t A_BYTES = 128u * CIN * 2u, B_BYTES = (uint32_t)NP * CIN * 2u;
    constexpr uint32_t TCOLS = NP <= 32 ? 32 : NP <= 64 ? 64 : NP <= 128 ? 128 : 256;
    constexpr uint32_t IDESC = tc::idesc_bf16(128, NP);
    __shared__ __align__(128) uint8_t sa[S][A_BYTES];
    __shared__ __align__(128) uint8_t sb[S][B_BYTES];
    __shared__ __align__(8) uint64_t bar[S];
    __shared__ uint32_t tmem_slot;
    const int V = nd * nd * nd, nbase = (int)blockIdx.y * NP;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    if (tid == 0) {
        for (int i = 0; i < S; i++) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc::saddr(&bar[i])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc::saddr(&tmem_slot)),
                     "r"(TCOLS) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    const int v = blockIdx.x * 128 + (int)tid;  // this thread's voxel (A row)
    const int x = v % nd, y = (v / nd) % nd, z = v / (nd * nd);
    // this thread's share of tap t's tiles; one cp.async group per call (empty past the last tap)
    auto load = [&](int t) {
        if (t < 27) {
            const int st = t % S;
            const int xx = x + dil * tap_off(t, 0), yy = y + dil * tap_off(t, 1), zz = z + dil * tap_off(t, 2);
            const bool in = v < V && xx >= 0 && yy >= 0 && zz >= 0 && xx < nd && yy < nd && zz < nd;
            const __nv_bfloat16* src = act + (size_t)(in ? xx + (yy + zz * nd) * nd : 0) * CIN;
            uint8_t* dst = sa[st] + (tid >> 3) * SBO + (tid & 7u) * 16u;
#pragma unroll
            for (uint32_t c = 0; c < KCOL; c++) cp_async16(dst + c * 128u, src + c * 8u, in ? 16u : 0u);
            for (uint32_t i = tid; i < (uint32_t)NP * KCOL; i += 128u) {
                const uint32_t n = i / KCOL, c = i % KCOL;
                const bool has = nbase + (int)n < Cout;
                cp_async16(sb[st] + (n >> 3) * SBO + c * 128u + (n & 7u) * 16u,
                           wkT + (has ? (size_t)(nbase + n) * K + t * CIN + c * 8u : 0), has ? 16u : 0u);
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
#pragma unroll 1
    for (int t = 0; t < S - 1; t++) load(t);
    bool ok = true;
    int last = -1;  // last tap whose MMAs were issued
#pragma unroll 1
    for (int t = 0; t < 27; t++) {
        const int st = t % S;
        asm volatile("cp.async.wait_group %0;" ::"n"(S - 2) : "memory");  // this thread's loads of tap t
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");     // generic writes -> tensor-core reads
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (uint32_t kk = 0; kk < KCOL / 2; kk++) {  // K = 16 per MMA = two core-matrix columns
                const uint64_t ad = tc::sdesc(tc::saddr(sa[st]) + kk * 256u, 128u, SBO);
                const uint64_t bd = tc::sdesc(tc::saddr(sb[st]) + kk * 256u, 128u, SBO);
                const uint32_t acc = (t > 0 || kk > 0) ? 1u : 0u;
                asm volatile("{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                             " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                             ::"r"(tmem), "l"(ad), "l"(bd), "r"(IDESC), "r"(acc) : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(tc::saddr(&bar[st])) : "memory");
        }
        last = t;
        // the stage of tap t - 1 takes tap t + S - 1 once the MMAs of tap t - 1 have read it
        if (t >= 1) ok = tc::wait(&bar[(t - 1) % S], (uint32_t)((t - 1) / S) & 1u);
        if (!__syncthreads_and(ok)) break;
        load(t + S - 1);
    }
    // the commit of the last tap covers every MMA issued before it
    if (last >= 0 && !tc::wait(&bar[last % S], (uint32_t)(last / S) & 1u)) ok = false;
    asm volatile("cp.async.wait_all;" ::: "memory");
    ok = __syncthreads_and(ok) != 0;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (ok) {
        const uint32_t row = tmem + ((warp * 32u) << 16);  // this warp's TMEM lanes
        const int vv = blockIdx.x * 128 + (int)(warp * 32u + lane);
#pragma unroll 1
        for (int c0 = 0; c0 < NP; c0 += 8) {
            uint32_t r[8];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7])
                         : "r"(row + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            const int n0 = nbase + c0;
            if (vv < V && n0 < Cout) {
                float val[8];
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const size_t o = (size_t)(n0 + e) * V + vv;
                    val[e] = __uint_as_float(r[e]);
                    if (n0 + e < Cout) {
                        if (res) val[e] += res[o];
                        if (out) out[o] = val[e];
                    }
                }
                if (outb) {
                    if (n0 + 8 <= Cout && Cout % 8 == 0) {  // one 16-byte store of 8 channels
                        uint4 pkd;
                        uint32_t* pw = (uint32_t*)&pkd;
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            const __nv_bfloat162 h2 = __floats2bfloat162_rn(val[2 * e], val[2 * e + 1]);
                            pw[e] = *(const uint32_t*)&h2;
                        }
                        *(uint4*)(outb + (size_t)vv * Cout + n0) = pkd;
                    } else {
                        for (int e = 0; e < 8 && n0 + e < Cout; e++) outb[(size_t)vv * Cout + n0 + e] = __float2bfloat16(val[e]);
                    }
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(err, 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TCOLS) : "memory");
}

// launch of one convolution layer on the tensor cores: Cout 32 in chunks of 16
// channels, the 168-channel head in chunks of 48 (more CTAs for the small grids)
void launch_conv_tc(const __nv_bfloat16* act, const __nv_bfloat16* wkT, const float* res, float* out,
                    __nv_bfloat16* outb, int cin, int cout, int dil, int nd, uint32_t* err, cudaStream_t s) {
    const unsigned gt = (unsigned)((nd * nd * nd + 127) / 128);
    if (cin == 16) k_conv_tc<16, 16, 4><<<dim3(gt, (cout + 15) / 16), 128, 0, s>>>(act, wkT, res, out, outb, cout, dil, nd, err);
    else if (cout <= 32) k_conv_tc<32, 16, 4><<<dim3(gt, (cout + 15) / 16), 128, 0, s>>>(act, wkT, res, out, outb, cout, dil, nd, err);
    else k_conv_tc<32, 48, 4><<<dim3(gt, (cout + 47) / 48), 128, 0, s>>>(act, wkT, res, out, outb, cout, dil, nd, err);
}

// network input in the inference layout: act [V][16] bf16, channels 4..15 zero
__global__ void k_input_bf16(const float* X, __nv_bfloat16* act, int V) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= V * 16) return;
    const int v = i / 16, c = i % 16;
    act[i] = __float2bfloat16(c < 4 ? X[(size_t)c * V + v] : 0.0f);
}

// ---------------------------------------------------------------------------
// self-test: the tcgen05 convolution against the mma.sync one on pseudo-random
// BF16 activations and weights (same products, FP32 accumulation in another
// order), max |diff| / max |reference| over FP32 outputs
// ---------------------------------------------------------------------------
__global__ void k_fill_bf16(__nv_bfloat16* p, size_t n, uint64_t seed) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t z = seed + i * 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    p[i] = __float2bfloat16((float)(z >> 40) * (1.0f / 8388608.0f) - 1.0f);
}

// wkT[co][tap * cinp + ci] = w[co][ci][tap] (zero for the padding channels ci >= cin)
__global__ void k_pack_weights(const float* w, __nv_bfloat16* wkT, int cin, int cinp, int cout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cout * 27 * cinp) return;
    const int co = i / (27 * cinp), k = i % (27 * cinp), tap = k / cinp, ci = k % cinp;
    wkT[i] = __float2bfloat16(ci < cin ? w[((size_t)co * cin + ci) * 27 + tap] : 0.0f);
}

// statistics of the current sources over the bins first..V-1: means q_m, J_m of q
// and of q v (FP64 sums), and the largest deviations from them.  scales[0] =
// max |q - q_m|, scales[1] = max over the three components of |q v - J_m| (1 where
// zero), scales[2] = q_m, scales[3..5] = J_m.
__global__ void k_source_scale(const float* qu_lod, int V, int first, float* scales) {
    __shared__ double r[4][256];
    __shared__ float mean[4];
    const float4* qu = (const float4*)qu_lod;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (int v = first + threadIdx.x; v < V; v += blockDim.x) {
        const float4 L = qu[v];
        s0 += L.x; s1 += L.x * L.y; s2 += L.x * L.z; s3 += L.x * L.w;
    }
    r[0][threadIdx.x] = s0; r[1][threadIdx.x] = s1; r[2][threadIdx.x] = s2; r[3][threadIdx.x] = s3;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off)
            for (int c = 0; c < 4; c++) r[c][threadIdx.x] += r[c][threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x < 4) mean[threadIdx.x] = V > first ? (float)(r[threadIdx.x][0] / (double)(V - first)) : 0.0f;
    __syncthreads();
    float mq = 0.0f, mv = 0.0f;
    for (int v = first + threadIdx.x; v < V; v += blockDim.x) {
        const float4 L = qu[v];
        mq = fmaxf(mq, fabsf(L.x - mean[0]));
        mv = fmaxf(mv, fmaxf(fabsf(L.x * L.y - mean[1]), fmaxf(fabsf(L.x * L.z - mean[2]), fabsf(L.x * L.w - mean[3]))));
    }
    __syncthreads();
    r[0][threadIdx.x] = mq;
    r[1][threadIdx.x] = mv;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            r[0][threadIdx.x] = fmax(r[0][threadIdx.x], r[0][threadIdx.x + off]);
            r[1][threadIdx.x] = fmax(r[1][threadIdx.x], r[1][threadIdx.x + off]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scales[0] = r[0][0] > 0.0 ? (float)r[0][0] : 1.0f;
        scales[1] = r[1][0] > 0.0 ? (float)r[1][0] : 1.0f;
        for (int c = 0; c < 4; c++) scales[2 + c] = mean[c];
    }
}

// ---------------------------------------------------------------------------
// per-cell field from the surrogate: exact near bins + interpolated far field.
// One thread block per bin, walking the bin's cells in tiles of SC_CELLS:
// all of them share the bin's list of near sources (shared memory, ascending
// bin order, built once) and its 27 x 6 node values.  Near sums use the FAST
// arithmetic in packed pairs (far_fast2).
//   Y [OUT_PAD][V] network output (normalised); scales: (sq, sv) from the device
// ---------------------------------------------------------------------------
constexpr uint32_t SC_CPT = 4, SC_THREADS = 256, SC_CELLS = SC_CPT * SC_THREADS;
struct SurSmem {
    FastSrc src[Surrogate::NEAR_CAND];
    float node[Surrogate::OUT_CH];
    // node values contracted along x: t1[lx][iy + 3 iz][c] = sum_ix wx_ix(lx) node[ix + 3 (iy + 3 iz)][c]
    float4 t1[Surrogate::MAX_BLOCK][9][2];
    // E_stat, B_stat of the tile's cells, fetched with cp.async while the near sums run
    float stat[6][SC_CELLS];
    // interpolation weights along y (wyz[0][ly]) and z (wyz[1][lz]) of the nodes 0, 1/2, 1
    float4 wyz[2][Surrogate::MAX_BLOCK];
    uint32_t count;
};


__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
                 : "memory");
}

__device__ __forceinline__ void quad_weights(float t, float* w) {  // Lagrange weights of the nodes 0, 1/2, 1
    w[0] = 2.0f * (t - 0.5f) * (t - 1.0f);
    w[1] = -4.0f * t * (t - 1.0f);
    w[2] = 2.0f * t * (t - 0.5f);
}

__device__ __forceinline__ void surrogate_tile(const DevLbm& L, SurSmem& sm, const float4* t2, uint32_t bin, int bx,
                                               int by, int bz, uint32_t tile, uint32_t cells, const Magic& mx,
                                               const Magic& mxy);

__global__ void __launch_bounds__(SC_THREADS, 2) k_surrogate_cells(const DevLbm L, const float* Y, const float* G,
                                                                const float* scales, float yE, float yB) {
    extern __shared__ __align__(16) uint8_t sur_smem[];  // SurSmem, then the t2 table
    SurSmem& sm = *reinterpret_cast<SurSmem*>(sur_smem);
    const uint32_t bin = blockIdx.x;
    const int nd = (int)L.nd, V = nd * nd * nd;
    const int bx = (int)bin % nd, by = ((int)bin / nd) % nd, bz = (int)bin / (nd * nd);
    if (threadIdx.x < 32) {  // near sources in ascending bin index (offsets in z, y, x order)
        const uint32_t lane = threadIdx.x;
        const float4* qu = (const float4*)L.qu_lod;
        uint32_t cnt = 0;
        constexpr int S = Surrogate::NEAR_SIDE, R = Surrogate::RNEAR;
        for (int o0 = 0; o0 < Surrogate::NEAR_CAND; o0 += 32) {
            const int o = o0 + (int)lane;
            const int x = bx + o % S - R, y = by + (o / S) % S - R, z = bz + o / (S * S) - R;
            const int d = x + (y + z * nd) * nd;
            const bool ok = o < Surrogate::NEAR_CAND && x >= 0 && y >= 0 && z >= 0 && x < nd && y < nd && z < nd && d != (int)bin &&
                            (uint32_t)d >= L.first_src;
            const uint32_t m = __ballot_sync(0xFFFFFFFFu, ok);
            if (ok) {  // coordinates relative to this bin's centre
                const float4 o = L.lod_pos[bin];
                fast_src(sm.src[cnt + __popc(m & ((1u << lane) - 1u))], L.lod_pos[d], qu[d], o.x, o.y, o.z, false);
            }
            cnt += __popc(m);
        }
        if (lane == 0) sm.count = cnt;
    }
    {  // node values in field units: network (fluctuations) + mean-source term
        const float sE = scales[0] * yE, sB = scales[1] * yB, qm = scales[2];
        const float jx = scales[3], jy = scales[4], jz = scales[5];
        for (uint32_t i = threadIdx.x; i < (uint32_t)Surrogate::OUT_CH; i += blockDim.x) {
            const uint32_t j6 = i - i % 6u, c = i % 6u;
            const float y = Y[(size_t)i * V + bin];
            const float gx = G[(size_t)j6 * V + bin], gy = G[(size_t)(j6 + 1) * V + bin], gz = G[(size_t)(j6 + 2) * V + bin];
            float v;
            if (c < 3u) v = fmaf(sE, y, qm * (c == 0u ? gx : c == 1u ? gy : gz));
            else v = fmaf(sB, y, c == 3u ? jy * gz - jz * gy : c == 4u ? jz * gx - jx * gz : jx * gy - jy * gx);
            sm.node[i] = v;
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < L.bsx * 9u * 8u; i += blockDim.x) {
        const uint32_t lx = i / 72u, jk = (i / 8u) % 9u, c = i % 8u;
        float wx[3];
        quad_weights(L.bsx > 1 ? (float)lx / (float)(L.bsx - 1) : 0.0f, wx);
        float v = 0.0f;
        if (c < 6u)
            for (int ix = 0; ix < 3; ix++) v = fmaf(wx[ix], sm.node[(ix + 3 * jk) * 6 + c], v);
        ((float*)&sm.t1[lx][jk][0])[c] = v;
    }
    for (uint32_t i = threadIdx.x; i < 2u * Surrogate::MAX_BLOCK; i += blockDim.x) {
        const uint32_t a = i / Surrogate::MAX_BLOCK, l = i % Surrogate::MAX_BLOCK, b = a == 0u ? L.bsy : L.bsz;
        float w[3];
        quad_weights(b > 1u ? (float)l / (float)(b - 1u) : 0.0f, w);
        sm.wyz[a][l] = make_float4(w[0], w[1], w[2], 0.0f);
    }
    __syncthreads();
    // contracted along y as well: t2[(ly bsx + lx) 3 + iz][c] = sum_iy wy_iy(ly) t1[lx][iy + 3 iz][c],
    // behind SurSmem in dynamic shared memory (bsx bsy 3 x 8 floats)
    float4* t2 = reinterpret_cast<float4*>(sur_smem + sizeof(SurSmem));
    for (uint32_t i = threadIdx.x; i < L.bsx * L.bsy * 24u; i += blockDim.x) {
        const uint32_t c = i % 8u, iz = (i / 8u) % 3u, lx = (i / 24u) % L.bsx, ly = i / (24u * L.bsx);
        const float4 wy = sm.wyz[0][ly];
        float v = 0.0f;
        if (c < 6u) {
            const float* t = (const float*)&sm.t1[lx][0][0];
            v = fmaf(wy.x, t[(0u + 3u * iz) * 8u + c], v);
            v = fmaf(wy.y, t[(1u + 3u * iz) * 8u + c], v);
            v = fmaf(wy.z, t[(2u + 3u * iz) * 8u + c], v);
        }
        ((float*)t2)[i] = v;
    }
    __syncthreads();

    const uint32_t cells = L.bsx * L.bsy * L.bsz;
    const Magic mx(L.bsx), mxy(L.bsx * L.bsy);
    for (uint32_t tile = 0; tile * SC_CELLS < cells; tile++) surrogate_tile(L, sm, t2, bin, bx, by, bz, tile, cells, mx, mxy);
}

__device__ __forceinline__ void surrogate_tile(const DevLbm& L, SurSmem& sm, const float4* t2, uint32_t bin, int bx,
                                               int by, int bz, uint32_t tile, uint32_t cells, const Magic& mx,
                                               const Magic& mxy) {
    // cell k of this thread: local index li -> (lx, ly, lz) in the bin, kept packed
    // (10 bits each) for the tail; flags are read now and used after the near sums
    float rx[SC_CPT], ry[SC_CPT], rz[SC_CPT];  // cell coordinates relative to the bin centre
    FarSums fs[SC_CPT / 2];
    uint32_t pc[SC_CPT], fl[SC_CPT];
    const size_t N = L.n;
    const float4 o = L.lod_pos[bin];
#pragma unroll
    for (uint32_t k = 0; k < SC_CPT; k++) {
        const uint32_t li = tile * SC_CELLS + threadIdx.x + k * SC_THREADS;
        const bool in = li < cells;
        const uint32_t lc = in ? li : 0u;
        const uint32_t lz = mxy.div(lc), r = lc - lz * mxy.d, ly = mx.div(r), lx = r - ly * mx.d;
        pc[k] = lx | ly << 10 | lz << 20;
        const uint32_t x = bx * L.bsx + lx, y = by * L.bsy + ly, z = bz * L.bsz + lz;
        const uint32_t m = x + (y + z * L.ny) * L.nx;
        fl[k] = F_S;
        if (in) {
            fl[k] = L.flags[m];
            // the static fields are needed after the near sums: copy them into this
            // thread's shared-memory slots now (only this thread reads them)
            const uint32_t slot = k * SC_THREADS + threadIdx.x;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                cp_async4(&sm.stat[c][slot], L.e_stat + c * N + m);
                cp_async4(&sm.stat[3 + c][slot], L.b_stat + c * N + m);
            }
        }
        rx[k] = (float)x - o.x; ry[k] = (float)y - o.y; rz[k] = (float)z - o.z;
    }
    Pair3 cp[SC_CPT / 2];
    P2 cc[SC_CPT / 2];
#pragma unroll
    for (uint32_t j = 0; j < SC_CPT / 2; j++) {
        cp[j] = {pk(rx[2 * j], rx[2 * j + 1]), pk(ry[2 * j], ry[2 * j + 1]), pk(rz[2 * j], rz[2 * j + 1])};
        cc[j] = pk(fmaf(rz[2 * j], rz[2 * j], fmaf(ry[2 * j], ry[2 * j], rx[2 * j] * rx[2 * j])),
                   fmaf(rz[2 * j + 1], rz[2 * j + 1], fmaf(ry[2 * j + 1], ry[2 * j + 1], rx[2 * j + 1] * rx[2 * j + 1])));
        far_zero(fs[j]);
    }
    const uint32_t cnt = sm.count;
    // the next source's values are read from shared memory while this one is summed
    FastSrc S = sm.src[0];
#pragma unroll 1
    for (uint32_t s = 0; s < cnt; s++) {
        const FastSrc Sn = sm.src[s + 1u < cnt ? s + 1u : s];
#pragma unroll
        for (uint32_t j = 0; j < SC_CPT / 2; j++) far_fast2(cp[j], cc[j], S, fs[j]);
        S = Sn;
    }
    asm volatile("cp.async.commit_group;\n cp.async.wait_group 0;" ::: "memory");
#pragma unroll
    for (uint32_t k = 0; k < SC_CPT; k++) {
        if ((fl[k] & F_BO) == F_S) continue;  // solid, or no cell
        const uint32_t lx = pc[k] & 1023u, ly = (pc[k] >> 10) & 1023u, lz = pc[k] >> 20;
        const uint32_t slot = k * SC_THREADS + threadIdx.x;
        const uint32_t m = (bx * L.bsx + lx) + ((by * L.bsy + ly) + (bz * L.bsz + lz) * L.ny) * L.nx;
        float e[3] = {0.0f, 0.0f, 0.0f}, b[3] = {0.0f, 0.0f, 0.0f};
        far_finish(cp[k / 2], fs[k / 2], (k & 1u) != 0, e, b);
        // triquadratic interpolation: the x and y contractions are tabulated per bin (t2)
        const float4 wz = sm.wyz[1][lz];
        const float wz3[3] = {wz.x, wz.y, wz.z};
        const float4* tc = t2 + (size_t)((ly * L.bsx + lx) * 3u) * 2u;
        float far[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int iz = 0; iz < 3; iz++) {
            const float4 a = tc[2 * iz], b2 = tc[2 * iz + 1];
            far[0] = fmaf(wz3[iz], a.x, far[0]); far[1] = fmaf(wz3[iz], a.y, far[1]); far[2] = fmaf(wz3[iz], a.z, far[2]);
            far[3] = fmaf(wz3[iz], a.w, far[3]); far[4] = fmaf(wz3[iz], b2.x, far[4]); far[5] = fmaf(wz3[iz], b2.y, far[5]);
        }
        L.e_dyn[m] = sm.stat[0][slot] + L.ke * (e[0] + far[0]);
        L.e_dyn[N + m] = sm.stat[1][slot] + L.ke * (e[1] + far[1]);
        L.e_dyn[2 * N + m] = sm.stat[2][slot] + L.ke * (e[2] + far[2]);
        L.b_dyn[m] = sm.stat[3][slot] + L.kmu * (b[0] + far[3]);
        L.b_dyn[N + m] = sm.stat[4][slot] + L.kmu * (b[1] + far[4]);
        L.b_dyn[2 * N + m] = sm.stat[5][slot] + L.kmu * (b[2] + far[5]);
    }
}

// ---------------------------------------------------------------------------
// sampled exact check: exact E/B (FAST arithmetic, full bin range) on `count`
// cells picked by a hash of the step, compared with the field values the
// surrogate wrote (E_stat + KE e, B_stat + KMU b: the values the next step
// uses).  stats[0] = max |dE|, [1] = max |E|, [2] = max |dB|, [3] = max |B|
// (as float bits, atomicMax on non-negative floats), [4] = 1 when an exact
// sample was non-finite
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

// |surrogate - exact| of one component.  Both finite: the difference.  Exactly
// one finite: a huge error (forces the fallback).  Both non-finite: 0 -- a
// non-finite source bin makes the exact sum non-finite in every cell, so the
// exact kernel would write a non-finite field as well and the fallback could
// not give a finite answer.
__device__ __forceinline__ float sample_diff(float sur, float exact) {
    const bool fs = isfinite(sur), fe = isfinite(exact);
    if (fs && fe) return fabsf(sur - exact);
    return fs == fe ? 0.0f : 3.0e38f;
}

// one warp per sampled cell: lanes take every 32nd bin, then a shuffle reduction
__global__ void __launch_bounds__(128) k_sample_check(const DevLbm L, uint32_t count, uint32_t salt, uint32_t* stats,
                                                     const unsigned long long* counters) {
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (i >= count) return;  // warp-uniform
    salt += (uint32_t)counters[0] * 0x9e3779b9u;  // a new sample set every step, also under graph replay
    uint32_t n = hash32(i * 2654435761u + salt) % L.n;
    for (int tries = 0; tries < 8 && (L.flags[n] & F_BO) == F_S; tries++) n = hash32(n + 0x9e3779b9u) % L.n;
    if ((L.flags[n] & F_BO) == F_S) return;  // warp-uniform
    uint32_t x, y, z;
    cell_xyz(L, n, x, y, z);
    const uint32_t own = x / L.bsx + (y / L.bsy + z / L.bsz * L.nd) * L.nd;
    float e[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    const float4* qu = (const float4*)L.qu_lod;
    const uint32_t last = src_last<true>(L);  // bins from 8^D on are always zero
    for (uint32_t d = L.first_src + lane; d < last; d += 32u) {
        if (d == own) continue;
        const float4 p = L.lod_pos[d], v = qu[d];
        add_src<true>((float)x - p.x, (float)y - p.y, (float)z - p.z, make_float4(v.x, v.x * v.y, v.x * v.z, v.x * v.w),
                      e, b);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            e[c] += __shfl_xor_sync(0xFFFFFFFFu, e[c], off);
            b[c] += __shfl_xor_sync(0xFFFFFFFFu, b[c], off);
        }
    if (lane != 0) return;
    const size_t N = L.n;
    float dE = 0.0f, mE = 0.0f, dB = 0.0f, mB = 0.0f;
    bool nonfinite = false;
    for (int c = 0; c < 3; c++) {
        const float ef = L.e_stat[c * N + n] + L.ke * e[c];
        const float bf = L.b_stat[c * N + n] + L.kmu * b[c];
        dE = fmaxf(dE, sample_diff(L.e_dyn[c * N + n], ef));
        dB = fmaxf(dB, sample_diff(L.b_dyn[c * N + n], bf));
        mE = fmaxf(mE, isfinite(ef) ? fabsf(ef) : 0.0f);
        mB = fmaxf(mB, isfinite(bf) ? fabsf(bf) : 0.0f);
        nonfinite |= !isfinite(ef) || !isfinite(bf);
    }
    atomicMax(&stats[0], __float_as_uint(dE));
    atomicMax(&stats[1], __float_as_uint(mE));
    atomicMax(&stats[2], __float_as_uint(dB));
    atomicMax(&stats[3], __float_as_uint(mB));
    if (nonfinite) atomicOr(&stats[4], 1u);
}

// decides the fallback on the device: flag = 1 when a relative error exceeds tol,
// or for good once a network convolution gave up waiting (stats[5], never cleared)
__global__ void k_sample_decide(uint32_t* stats, float tol, uint32_t* flag, float* last, unsigned long long* counters) {
    const float dE = __uint_as_float(stats[0]), mE = __uint_as_float(stats[1]);
    const float dB = __uint_as_float(stats[2]), mB = __uint_as_float(stats[3]);
    const float rE = mE > 0.0f ? dE / mE : dE, rB = mB > 0.0f ? dB / mB : dB;
    const bool bad = !(rE <= tol) || !(rB <= tol) || stats[5] != 0u;
    *flag = bad ? 1u : 0u;
    last[0] = rE;
    last[1] = rB;
    counters[0] += 1ull;
    if (bad) counters[1] += 1ull;
    if (stats[4]) counters[2] += 1ull;
    stats[0] = stats[1] = stats[2] = stats[3] = stats[4] = 0u;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {
struct LayerDef { int cin, cout, dil; };
const LayerDef kLayers[10] = {{4, 32, 1}, {32, 32, 1}, {32, 32, 2}, {32, 32, 2}, {32, 32, 4},
                              {32, 32, 4}, {32, 32, 8}, {32, 32, 1}, {32, 32, 1}, {32, Surrogate::OUT_PAD, 1}};
unsigned blocks_for(size_t n, unsigned b) { return (unsigned)((n + b - 1) / b); }
}  // namespace

Surrogate::~Surrogate() {
    for (void* p : allocs_) cudaFree(p);
}

int Surrogate::alloc(void** p, size_t bytes) {
    if (cudaMalloc(p, bytes) != cudaSuccess) {
        cudaGetLastError();
        return ION_E_NOMEM;
    }
    allocs_.push_back(*p);
    cudaMemset(*p, 0, bytes);
    return ION_OK;
}

int Surrogate::init(int nd, float bsx, float bsy, float bsz, int first_src) {
    nd_ = nd;
    V_ = nd * nd * nd;
    bs_[0] = bsx; bs_[1] = bsy; bs_[2] = bsz;
    first_ = first_src;
    size_t off = 0;
    for (int l = 0; l < 10; l++) {
        woff_[l] = off;
        off += (size_t)kLayers[l].cin * kLayers[l].cout * 27;
    }
    nw_ = off;
    off = 0;
    for (int l = 0; l < 10; l++) {
        wkoff_[l] = off;
        off += (size_t)kLayers[l].cout * 27 * (kLayers[l].cin < 16 ? 16 : kLayers[l].cin);
    }
    nwk_ = off;
    int rc = 0;
    rc |= alloc((void**)&w_, nw_ * 4);
    rc |= alloc((void**)&gw_, nw_ * 4);
    rc |= alloc((void**)&m_, nw_ * 4);
    rc |= alloc((void**)&v_, nw_ * 4);
    rc |= alloc((void**)&wt_, (size_t)32 * OUT_PAD * 27 * 4);
    rc |= alloc((void**)&wk_, nwk_ * 2);
    rc |= alloc((void**)&scales_, 8 * 4);
    rc |= alloc((void**)&gunit_, (size_t)OUT_PAD * V_ * 4);
    rc |= alloc((void**)&stats_, 8 * 4);
    rc |= alloc((void**)&flag_, 4);
    rc |= alloc((void**)&last_, 2 * 4);
    rc |= alloc((void**)&counters_, 3 * 8);
    rc |= alloc((void**)&xin_, (size_t)4 * V_ * 4);
    rc |= alloc((void**)&yout_, (size_t)OUT_PAD * V_ * 4);
    rc |= alloc((void**)&ha_, (size_t)32 * V_ * 4);
    rc |= alloc((void**)&ab_, (size_t)32 * V_ * 2);
    rc |= alloc((void**)&bb_, (size_t)32 * V_ * 2);
    rc |= alloc((void**)&xb_, (size_t)16 * V_ * 2);
    if (rc) return ION_E_NOMEM;
    if (cudaFuncSetAttribute(k_surrogate_cells, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(SurSmem) + (size_t)MAX_BLOCK * MAX_BLOCK * 96u)) !=
        cudaSuccess)
        return ION_E_CUDA;
    // far field of a unit charge in every source bin at the 27 nodes: the field of
    // the mean sources (E = q_m G, B = J_m x G), exact and fixed by the geometry
    {
        std::vector<float> one((size_t)4 * V_, 0.0f);
        for (int v = first_; v < V_; v++) one[v] = 1.0f;
        if (cudaMemcpy(xin_, one.data(), one.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) return ION_E_CUDA;
        k_far_targets<<<blocks_for((size_t)V_ * NODES, 256), 256>>>(xin_, nd_, bs_[0], bs_[1], bs_[2], RNEAR, gunit_, 1);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return ION_E_CUDA;
    }
    return reset_weights(seed_);
}

// He-style initialisation scaled down so the residual stack starts near identity
int Surrogate::reset_weights(uint64_t seed) {
    std::mt19937_64 gen(seed);
    std::vector<float> w(nw_);
    for (int l = 0; l < 10; l++) {
        const float sd = (l >= 1 && l <= 8 ? 0.1f : 1.0f) / std::sqrt((float)kLayers[l].cin * 27.0f);
        std::normal_distribution<float> nd1(0.0f, sd);
        for (size_t i = 0; i < (size_t)kLayers[l].cin * kLayers[l].cout * 27; i++) w[woff_[l] + i] = nd1(gen);
    }
    ready_ = false;
    return cudaMemcpy(w_, w.data(), nw_ * 4, cudaMemcpyHostToDevice) == cudaSuccess ? ION_OK : ION_E_CUDA;
}

// FP32 forward of a batch; acts: 9 activation buffers [B][32][V] + output [B][OUT_PAD][V]
void Surrogate::forward_fp32(const float* X, int B, std::vector<float*>& acts, float* Y, cudaStream_t s) {
    auto conv = [&](const float* in, int l, const float* res, float* out) {
        const LayerDef& d = kLayers[l];
        dim3 grid(blocks_for((size_t)B * V_, 128), (d.cout + COG - 1) / COG);
        k_conv_fwd<<<grid, 128, 0, s>>>(in, w_ + woff_[l], res, out, d.cin, d.cout, d.dil, nd_, B);
    };
    // acts: h0, t0, h1, t1, h2, t2, h3, t3, h4
    conv(X, 0, nullptr, acts[0]);
    for (int i = 0; i < 4; i++) {
        conv(acts[2 * i], 1 + 2 * i, nullptr, acts[2 * i + 1]);
        conv(acts[2 * i + 1], 2 + 2 * i, acts[2 * i], acts[2 * i + 2]);
    }
    conv(acts[8], 9, nullptr, Y);
}

void Surrogate::backward_fp32(const float* X, int B, std::vector<float*>& acts, const float* gY, std::vector<float*>& g,
                              cudaStream_t s) {
    // g: two gradient buffers [B][32][V] used alternately
    auto wgrad = [&](const float* in, const float* gout, int l) {
        const LayerDef& d = kLayers[l];
        k_conv_wgrad<<<d.cin * d.cout, 256, 0, s>>>(in, gout, gw_ + woff_[l], d.cin, d.cout, d.dil, nd_, B);
    };
    auto dgrad = [&](const float* gout, int l, const float* res, float* gin) {  // gin = res + conv^T(gout)
        const LayerDef& d = kLayers[l];
        k_transpose_flip<<<blocks_for((size_t)d.cin * d.cout * 27, 256), 256, 0, s>>>(w_ + woff_[l], wt_, d.cin, d.cout);
        dim3 grid(blocks_for((size_t)B * V_, 128), (d.cin + COG - 1) / COG);
        k_conv_fwd<<<grid, 128, 0, s>>>(gout, wt_, res, gin, d.cout, d.cin, d.dil, nd_, B);
    };
    float* gh = g[0];
    float* gt = g[1];
    float* gtmp = g[2];
    wgrad(acts[8], gY, 9);
    dgrad(gY, 9, nullptr, gh);  // dL/dh4
    for (int i = 3; i >= 0; i--) {
        // h_{i+1} = h_i + conv_b(t_i), t_i = conv_a(h_i)
        wgrad(acts[2 * i + 1], gh, 2 + 2 * i);
        dgrad(gh, 2 + 2 * i, nullptr, gt);            // dL/dt_i
        wgrad(acts[2 * i], gt, 1 + 2 * i);
        dgrad(gt, 1 + 2 * i, gh, gtmp);               // dL/dh_i = dL/dh_{i+1} + conv_a^T(dL/dt_i)
        std::swap(gh, gtmp);
    }
    wgrad(X, gh, 0);
    g[0] = gh;
    g[2] = gtmp;
}

// One training snapshot of the network input, x [4][V]: the fluctuations of the bin
// sources about their means (the means' field is exact, outside the network).
// Each channel is a random mix of up to three plane waves of wavenumber <= 2 per
// axis, a Gaussian charge cloud and white noise, minus its mean over the source
// bins, then divided by its largest deviation like the inference input (charge
// alone; current by the largest of its three components).  Bins below first_src
// carry no sources.
void Surrogate::make_snapshot(std::mt19937_64& gen, float* x) const {
    std::uniform_real_distribution<float> U(-1.0f, 1.0f), P(0.0f, 1.0f);
    std::uniform_int_distribution<int> K(0, 2);
    const int nd = nd_;
    const float tau = 6.28318530717958647692f;
    for (int c = 0; c < 4; c++) {
        float* xc = x + (size_t)c * V_;
        const int waves = P(gen) < 0.6f ? 1 + (int)(P(gen) * 3.0f) : 0;
        float wk[3][3], wa[3], wp[3];
        for (int w = 0; w < waves; w++) {
            for (int d = 0; d < 3; d++) wk[w][d] = (float)K(gen);
            wa[w] = U(gen);
            wp[w] = tau * P(gen);
        }
        const bool blob = P(gen) < 0.4f;
        const float bc[3] = {nd * P(gen), nd * P(gen), nd * P(gen)}, bw = 1.0f + 3.0f * P(gen), ba = U(gen);
        const float white = P(gen) < 0.3f ? 1.0f : 0.05f + 0.5f * P(gen);
        for (int v = 0; v < V_; v++) {
            if (v < first_) { xc[v] = 0.0f; continue; }
            const float px = (float)(v % nd), py = (float)((v / nd) % nd), pz = (float)(v / (nd * nd));
            float val = white * U(gen);
            for (int w = 0; w < waves; w++)
                val += wa[w] * std::cos(tau * (wk[w][0] * px + wk[w][1] * py + wk[w][2] * pz) / (float)nd + wp[w]);
            if (blob) {
                const float r2 = (px - bc[0]) * (px - bc[0]) + (py - bc[1]) * (py - bc[1]) + (pz - bc[2]) * (pz - bc[2]);
                val += ba * std::exp(-0.5f * r2 / (bw * bw));
            }
            xc[v] = val;
        }
        double mean = 0.0;
        for (int v = first_; v < V_; v++) mean += xc[v];
        mean /= std::max(V_ - first_, 1);
        for (int v = first_; v < V_; v++) xc[v] -= (float)mean;
    }
    float mq = 0.0f, mv = 0.0f;
    for (int v = 0; v < V_; v++) {
        mq = std::max(mq, std::fabs(x[v]));
        for (int c = 1; c < 4; c++) mv = std::max(mv, std::fabs(x[(size_t)c * V_ + v]));
    }
    for (int v = 0; v < V_; v++) {
        if (mq > 0.0f) x[v] /= mq;
        for (int c = 1; c < 4; c++)
            if (mv > 0.0f) x[(size_t)c * V_ + v] /= mv;
    }
}

int Surrogate::train(int nsamples, int epochs, int batch, float lr, uint64_t seed, cudaStream_t s, float* rel_err) {
    // every training starts from the same initial weights (a function of the seed)
    if (int rc = reset_weights(seed ^ 0x5EEDu)) return rc;
    // training snapshots: random charge and current per bin, exact far-field targets
    const size_t xs = (size_t)4 * V_, ys = (size_t)OUT_PAD * V_;
    float *X = nullptr, *T = nullptr;
    if (cudaMalloc(&X, xs * nsamples * 4) != cudaSuccess || cudaMalloc(&T, ys * nsamples * 4) != cudaSuccess) {
        cudaFree(X);
        cudaGetLastError();
        return ION_E_NOMEM;
    }
    {
        std::mt19937_64 gen(seed);
        std::vector<float> h(xs * nsamples);
        for (int sidx = 0; sidx < nsamples; sidx++) make_snapshot(gen, h.data() + sidx * xs);
        cudaMemcpy(X, h.data(), h.size() * 4, cudaMemcpyHostToDevice);
    }
    cudaMemsetAsync(T, 0, ys * nsamples * 4, s);  // padding channels stay zero
    k_far_targets<<<blocks_for((size_t)V_ * NODES * nsamples, 256), 256, 0, s>>>(X, nd_, bs_[0], bs_[1], bs_[2], RNEAR, T,
                                                                              nsamples);
    // normalisation of the E and B channel groups
    std::vector<float> th(ys * std::min(nsamples, 64));
    cudaMemcpyAsync(th.data(), T, th.size() * 4, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    double se = 0, sb = 0;
    size_t ne = 0, nb = 0;
    for (size_t i = 0; i < th.size(); i++) {
        const int chan = (int)((i / V_) % OUT_PAD);
        if (chan >= OUT_CH) continue;  // padding channels
        if (chan % 6 < 3) { se += (double)th[i] * th[i]; ne++; } else { sb += (double)th[i] * th[i]; nb++; }
    }
    yE_ = (float)std::sqrt(se / std::max<size_t>(ne, 1));
    yB_ = (float)std::sqrt(sb / std::max<size_t>(nb, 1));
    if (!(yE_ > 0)) yE_ = 1.0f;
    if (!(yB_ > 0)) yB_ = 1.0f;
    k_scale_targets<<<blocks_for(ys * nsamples, 256), 256, 0, s>>>(T, V_, ys * nsamples, 1.0f / yE_, 1.0f / yB_);
    // activations and gradients for one batch
    std::vector<float*> acts(9), g(3);
    float *Yb = nullptr, *gY = nullptr, *loss = nullptr;
    bool ok = true;
    for (auto& p : acts) ok &= cudaMalloc(&p, (size_t)batch * 32 * V_ * 4) == cudaSuccess;
    for (auto& p : g) ok &= cudaMalloc(&p, (size_t)batch * 32 * V_ * 4) == cudaSuccess;
    ok &= cudaMalloc(&Yb, (size_t)batch * ys * 4) == cudaSuccess;
    ok &= cudaMalloc(&gY, (size_t)batch * ys * 4) == cudaSuccess;
    ok &= cudaMalloc(&loss, 4) == cudaSuccess;
    int rc = ok ? ION_OK : ION_E_NOMEM;
    const int ntrain = std::max(1, nsamples - std::max(1, nsamples / 10));
    int t = 0;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    cudaMemsetAsync(m_, 0, nw_ * 4, s);
    cudaMemsetAsync(v_, 0, nw_ * 4, s);
    loss_.clear();
    // divergence guard: the weights of the best epoch are kept; an epoch whose
    // loss is not finite or above 4x the best restores them, clears the Adam
    // moments and halves the learning rate from then on
    float* wbest = nullptr;
    if (!rc && cudaMalloc(&wbest, nw_ * 4) != cudaSuccess) rc = ION_E_NOMEM;
    if (!rc) cudaMemcpyAsync(wbest, w_, nw_ * 4, cudaMemcpyDeviceToDevice, s);
    double best = 1e300;
    float lr_scale = 1.0f;
    for (int ep = 0; ep < epochs && !rc; ep++) {
        const float lr_ep = lr_scale * lr * (ep < epochs / 2 ? 1.0f : ep < 3 * epochs / 4 ? 0.3f : 0.1f);
        double ep_loss = 0.0;
        int nb_ = 0;
        for (int b0 = 0; b0 + batch <= ntrain; b0 += batch) {
            forward_fp32(X + (size_t)b0 * xs, batch, acts, Yb, s);
            cudaMemsetAsync(loss, 0, 4, s);
            k_mse<<<256, 256, 0, s>>>(Yb, T + (size_t)b0 * ys, gY, loss, (size_t)batch * ys);
            backward_fp32(X + (size_t)b0 * xs, batch, acts, gY, g, s);
            t++;
            const float c1 = 1.0f - std::pow(b1, (float)t), c2 = 1.0f - std::pow(b2, (float)t);
            k_adam<<<blocks_for(nw_, 256), 256, 0, s>>>(w_, gw_, m_, v_, nw_, lr_ep, b1, b2, eps, c1, c2);
            float lh = 0;
            cudaMemcpyAsync(&lh, loss, 4, cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            ep_loss += lh / ((double)batch * ys);
            nb_++;
        }
        const double el = ep_loss / std::max(nb_, 1);
        loss_.push_back((float)el);
        if (cudaGetLastError() != cudaSuccess) rc = ION_E_CUDA;
        if (std::isfinite(el) && el < best) {
            best = el;
            cudaMemcpyAsync(wbest, w_, nw_ * 4, cudaMemcpyDeviceToDevice, s);
        } else if (!std::isfinite(el) || el > 4.0 * best) {
            cudaMemcpyAsync(w_, wbest, nw_ * 4, cudaMemcpyDeviceToDevice, s);
            cudaMemsetAsync(m_, 0, nw_ * 4, s);
            cudaMemsetAsync(v_, 0, nw_ * 4, s);
            lr_scale *= 0.5f;
        }
    }
    if (!rc && !(loss_.empty()) && !(loss_.back() <= best)) cudaMemcpyAsync(w_, wbest, nw_ * 4, cudaMemcpyDeviceToDevice, s);
    cudaFree(wbest);
    // held-out error of the FP32 network and of the BF16 inference path
    if (!rc) {
        pack_bf16(s);
        double num32 = 0, num16 = 0, den = 0;
        std::vector<float> y32(ys), y16(ys), tt(ys);
        for (int sidx = ntrain; sidx < nsamples; sidx++) {
            forward_fp32(X + (size_t)sidx * xs, 1, acts, Yb, s);
            cudaMemcpyAsync(y32.data(), Yb, ys * 4, cudaMemcpyDeviceToHost, s);
            infer_bf16(X + (size_t)sidx * xs, s);
            cudaMemcpyAsync(y16.data(), yout_, ys * 4, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(tt.data(), T + (size_t)sidx * ys, ys * 4, cudaMemcpyDeviceToHost, s);
            cudaStreamSynchronize(s);
            for (size_t i = 0; i < ys; i++) {
                num32 += (double)(y32[i] - tt[i]) * (y32[i] - tt[i]);
                num16 += (double)(y16[i] - tt[i]) * (y16[i] - tt[i]);
                den += (double)tt[i] * tt[i];
            }
        }
        rel32_ = (float)std::sqrt(num32 / std::max(den, 1e-30));
        rel16_ = (float)std::sqrt(num16 / std::max(den, 1e-30));
        if (rel_err) *rel_err = rel16_;
        ready_ = true;
    }
    for (auto p : acts) cudaFree(p);
    for (auto p : g) cudaFree(p);
    cudaFree(Yb); cudaFree(gY); cudaFree(loss); cudaFree(X); cudaFree(T);
    return rc ? rc : (cudaGetLastError() == cudaSuccess ? ION_OK : ION_E_CUDA);
}

void Surrogate::pack_bf16(cudaStream_t s) {
    for (int l = 0; l < 10; l++) {
        const LayerDef& d = kLayers[l];
        const int cinp = d.cin < 16 ? 16 : d.cin;
        k_pack_weights<<<blocks_for((size_t)d.cout * 27 * cinp, 256), 256, 0, s>>>(w_ + woff_[l], wk_ + wkoff_[l], d.cin,
                                                                                    cinp, d.cout);
    }
}

// BF16 tensor-core forward of one sample X [4][V] (fp32) -> yout_ [OUT_PAD][V]
void Surrogate::infer_bf16(const float* X, cudaStream_t s) {
    // residual stream h in fp32 (ha_), bf16 voxel-major copies for the next conv (xb_/ab_/bb_);
    // a tcgen05 wait that gives up sets stats_[5], which forces the exact fallback
    k_input_bf16<<<blocks_for((size_t)16 * V_, 256), 256, 0, s>>>(X, xb_, V_);
    auto conv = [&](const __nv_bfloat16* in, int l, const float* res, float* out, __nv_bfloat16* outb) {
        const LayerDef& d = kLayers[l];
        launch_conv_tc(in, wk_ + wkoff_[l], res, out, outb, d.cin < 16 ? 16 : d.cin, d.cout, d.dil, nd_, stats_ + 5, s);
    };
    conv(xb_, 0, nullptr, ha_, ab_);  // h0
    for (int i = 0; i < 4; i++) {
        conv(ab_, 1 + 2 * i, nullptr, nullptr, bb_);  // t_i (bf16 only)
        conv(bb_, 2 + 2 * i, ha_, ha_, ab_);          // h_{i+1} = h_i + conv(t_i)
    }
    conv(ab_, 9, nullptr, yout_, nullptr);
}

void Surrogate::step(const DevLbm& L, cudaStream_t s, uint32_t salt) {
    k_source_scale<<<1, 256, 0, s>>>(L.qu_lod, V_, first_, scales_);
    k_pack_input_dev(L, s);
    infer_bf16(xin_, s);
    k_surrogate_cells<<<L.n_bins, SC_THREADS, sizeof(SurSmem) + (size_t)L.bsx * L.bsy * 96u, s>>>(L, yout_, gunit_,
                                                                                                 scales_, yE_, yB_);
    k_sample_check<<<blocks_for((size_t)check_cells_ * 32, 128), 128, 0, s>>>(L, check_cells_, salt, stats_, counters_);
    k_sample_decide<<<1, 1, 0, s>>>(stats_, tol_, flag_, last_, counters_);
}

// network input from the LOD table: X[c][v] = (q - q_m, q vx - J_m,x, q vy - J_m,y,
// q vz - J_m,z) divided by the step's deviation scales (the fluctuations about the
// source means); bins below first_src are no sources (sim_kernels.cl:943)
__global__ void k_pack_input_scaled(const float* qu_lod, int V, int first, const float* scales, float* X) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const float4 L = ((const float4*)qu_lod)[v];
    const bool use = v >= first;
    const float sq = scales[0], sv = scales[1];
    X[v] = use ? (L.x - scales[2]) / sq : 0.0f;
    X[V + v] = use ? (L.x * L.y - scales[3]) / sv : 0.0f;
    X[2 * V + v] = use ? (L.x * L.z - scales[4]) / sv : 0.0f;
    X[3 * V + v] = use ? (L.x * L.w - scales[5]) / sv : 0.0f;
}

void Surrogate::k_pack_input_dev(const DevLbm& L, cudaStream_t s) {
    k_pack_input_scaled<<<blocks_for(V_, 256), 256, 0, s>>>(L.qu_lod, V_, first_, scales_, xin_);
}

uint32_t Surrogate::launches_per_step() const { return 2 + 11 + 3; }  // scale, pack, 11 inference, cells, check, decide

int Surrogate::get_weights(float* host) const {
    return cudaMemcpy(host, w_, nw_ * 4, cudaMemcpyDeviceToHost) == cudaSuccess ? ION_OK : ION_E_CUDA;
}

int Surrogate::set_weights(const float* host, cudaStream_t s) {
    if (cudaMemcpy(w_, host, nw_ * 4, cudaMemcpyHostToDevice) != cudaSuccess) return ION_E_CUDA;
    pack_bf16(s);
    ready_ = true;
    return cudaStreamSynchronize(s) == cudaSuccess ? ION_OK : ION_E_CUDA;
}

int Surrogate::grad(const float* hX, const float* hT, int B, float* hloss, float* hgrad, cudaStream_t s) {
    const size_t xs = (size_t)4 * V_, ys = (size_t)OUT_PAD * V_;
    std::vector<float*> acts(9), g(3);
    float *X = nullptr, *T = nullptr, *Y = nullptr, *gY = nullptr, *loss = nullptr;
    bool ok = cudaMalloc(&X, xs * B * 4) == cudaSuccess && cudaMalloc(&T, ys * B * 4) == cudaSuccess &&
              cudaMalloc(&Y, ys * B * 4) == cudaSuccess && cudaMalloc(&gY, ys * B * 4) == cudaSuccess &&
              cudaMalloc(&loss, 4) == cudaSuccess;
    for (auto& p : acts) ok = ok && cudaMalloc(&p, (size_t)B * 32 * V_ * 4) == cudaSuccess;
    for (auto& p : g) ok = ok && cudaMalloc(&p, (size_t)B * 32 * V_ * 4) == cudaSuccess;
    int rc = ok ? ION_OK : ION_E_NOMEM;
    if (!rc) {
        cudaMemcpyAsync(X, hX, xs * B * 4, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(T, hT, ys * B * 4, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(loss, 0, 4, s);
        forward_fp32(X, B, acts, Y, s);
        k_mse<<<256, 256, 0, s>>>(Y, T, gY, loss, (size_t)B * ys);
        backward_fp32(X, B, acts, gY, g, s);
        cudaMemcpyAsync(hgrad, gw_, nw_ * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hloss, loss, 4, cudaMemcpyDeviceToHost, s);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) rc = ION_E_CUDA;
        *hloss /= (float)(ys * B);  // mean squared error, the loss whose gradient k_mse forms
    }
    for (auto p : acts) cudaFree(p);
    for (auto p : g) cudaFree(p);
    cudaFree(X); cudaFree(T); cudaFree(Y); cudaFree(gY); cudaFree(loss);
    cudaGetLastError();
    return rc;
}

int Surrogate::targets(const float* hX, float* hT, int B, cudaStream_t s) {
    const size_t xs = (size_t)4 * V_, ys = (size_t)OUT_PAD * V_;
    float *X = nullptr, *T = nullptr;
    int rc = cudaMalloc(&X, xs * B * 4) == cudaSuccess && cudaMalloc(&T, ys * B * 4) == cudaSuccess ? ION_OK
                                                                                                  : ION_E_NOMEM;
    if (!rc) {
        cudaMemcpyAsync(X, hX, xs * B * 4, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(T, 0, ys * B * 4, s);
        k_far_targets<<<blocks_for((size_t)V_ * NODES * B, 256), 256, 0, s>>>(X, nd_, bs_[0], bs_[1], bs_[2], RNEAR, T,
                                                                               B);
        cudaMemcpyAsync(hT, T, ys * B * 4, cudaMemcpyDeviceToHost, s);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) rc = ION_E_CUDA;
    }
    cudaFree(X);
    cudaFree(T);
    cudaGetLastError();
    return rc;
}

int Surrogate::forward(const float* hX, float* hY, bool bf16, cudaStream_t s) {
    const size_t xs = (size_t)4 * V_, ys = (size_t)OUT_PAD * V_;
    std::vector<float*> acts(9);
    float *X = nullptr, *Y = nullptr;
    bool ok = cudaMalloc(&X, xs * 4) == cudaSuccess && cudaMalloc(&Y, ys * 4) == cudaSuccess;
    for (auto& p : acts) ok = ok && cudaMalloc(&p, (size_t)32 * V_ * 4) == cudaSuccess;
    int rc = ok ? ION_OK : ION_E_NOMEM;
    if (!rc) {
        cudaMemcpyAsync(X, hX, xs * 4, cudaMemcpyHostToDevice, s);
        if (bf16) {
            infer_bf16(X, s);
            cudaMemcpyAsync(hY, yout_, ys * 4, cudaMemcpyDeviceToHost, s);
        } else {
            forward_fp32(X, 1, acts, Y, s);
            cudaMemcpyAsync(hY, Y, ys * 4, cudaMemcpyDeviceToHost, s);
        }
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) rc = ION_E_CUDA;
    }
    for (auto p : acts) cudaFree(p);
    cudaFree(X); cudaFree(Y);
    cudaGetLastError();
    return rc;
}

int Surrogate::save(const char* path) const {
    std::vector<float> w(nw_);
    if (cudaMemcpy(w.data(), w_, nw_ * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return ION_E_CUDA;
    FILE* f = fopen(path, "wb");
    if (!f) return ION_E_IO;
    const uint32_t hdr[4] = {0x474f5253u /* "SROG" */, 2u, (uint32_t)nd_, (uint32_t)nw_};
    bool ok = fwrite(hdr, 4, 4, f) == 4 && fwrite(&yE_, 4, 1, f) == 1 && fwrite(&yB_, 4, 1, f) == 1 &&
              fwrite(w.data(), 4, nw_, f) == nw_;
    fclose(f);
    return ok ? ION_OK : ION_E_IO;
}

int Surrogate::load(const char* path, cudaStream_t s) {
    FILE* f = fopen(path, "rb");
    if (!f) return ION_E_IO;
    uint32_t hdr[4];
    std::vector<float> w(nw_);
    bool ok = fread(hdr, 4, 4, f) == 4 && hdr[0] == 0x474f5253u && hdr[1] == 2u && hdr[2] == (uint32_t)nd_ &&
              hdr[3] == (uint32_t)nw_ && fread(&yE_, 4, 1, f) == 1 && fread(&yB_, 4, 1, f) == 1 &&
              fread(w.data(), 4, nw_, f) == nw_;
    fclose(f);
    if (!ok) return ION_E_FORMAT;
    if (cudaMemcpy(w_, w.data(), nw_ * 4, cudaMemcpyHostToDevice) != cudaSuccess) return ION_E_CUDA;
    pack_bf16(s);
    ready_ = true;
    return ION_OK;
}

int conv_tc_selftest(int nd, int cin, int cout, int dil, uint64_t seed, float* max_rel, cudaStream_t s) {
    if (nd < 4 || (nd * nd * nd) % 128 != 0 || !(cin == 16 || cin == 32) || !(cout == 32 || cout == 168) ||
        (cin == 16 && cout != 32))
        return ION_E_INVALID;
    const int V = nd * nd * nd, K = 27 * cin;
    __nv_bfloat16 *act = nullptr, *w = nullptr, *ob1 = nullptr, *ob2 = nullptr;
    float *o1 = nullptr, *o2 = nullptr;
    uint32_t* err = nullptr;
    bool ok = cudaMalloc(&act, (size_t)V * cin * 2) == cudaSuccess && cudaMalloc(&w, (size_t)cout * K * 2) == cudaSuccess &&
              cudaMalloc(&o1, (size_t)cout * V * 4) == cudaSuccess && cudaMalloc(&o2, (size_t)cout * V * 4) == cudaSuccess &&
              cudaMalloc(&ob1, (size_t)cout * V * 2) == cudaSuccess && cudaMalloc(&ob2, (size_t)cout * V * 2) == cudaSuccess &&
              cudaMalloc(&err, 4) == cudaSuccess;
    int rc = ok ? ION_OK : ION_E_NOMEM;
    if (!rc) {
        cudaMemsetAsync(err, 0, 4, s);
        k_fill_bf16<<<blocks_for((size_t)V * cin, 256), 256, 0, s>>>(act, (size_t)V * cin, seed);
        k_fill_bf16<<<blocks_for((size_t)cout * K, 256), 256, 0, s>>>(w, (size_t)cout * K, seed ^ 0xabcdefull);
        const unsigned gx = blocks_for((size_t)(V / 16) * 32, 128);
        if (cin == 16) {
            k_conv_bf16<16, 1><<<dim3(gx, cout / 8), 128, 0, s>>>(act, w, nullptr, o1, ob1, cout, dil, nd);
        } else if (cout == 32) {
            k_conv_bf16<32, 1><<<dim3(gx, 4), 128, 0, s>>>(act, w, nullptr, o1, ob1, cout, dil, nd);
        } else {
            k_conv_bf16<32, 1><<<dim3(gx, 21), 128, 0, s>>>(act, w, nullptr, o1, ob1, cout, dil, nd);
        }
        launch_conv_tc(act, w, nullptr, o2, ob2, cin, cout, dil, nd, err, s);
        std::vector<float> h1((size_t)cout * V), h2((size_t)cout * V);
        std::vector<__nv_bfloat16> b1((size_t)cout * V), b2((size_t)cout * V);
        uint32_t herr = 0;
        cudaMemcpyAsync(h1.data(), o1, h1.size() * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(h2.data(), o2, h2.size() * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(b1.data(), ob1, b1.size() * 2, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(b2.data(), ob2, b2.size() * 2, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) rc = ION_E_CUDA;
        else if (herr) rc = ION_E_TIMEOUT;
        else {
            double dmax = 0.0, rmax = 0.0;
            for (size_t i = 0; i < h1.size(); i++) {
                dmax = std::max(dmax, (double)std::fabs(h1[i] - h2[i]));
                rmax = std::max(rmax, (double)std::fabs(h1[i]));
                // the voxel-major BF16 copies (the next layer's input) as well
                dmax = std::max(dmax, (double)std::fabs(__bfloat162float(b1[i]) - __bfloat162float(b2[i])));
            }
            // an all-zero reference output would make any comparison pass
            *max_rel = rmax > 0.0 ? (float)(dmax / rmax) : INFINITY;
        }
    }
    cudaFree(act); cudaFree(w); cudaFree(o1); cudaFree(o2); cudaFree(ob1); cudaFree(ob2); cudaFree(err);
    cudaGetLastError();
    return rc;
}

}  // namespace ion
