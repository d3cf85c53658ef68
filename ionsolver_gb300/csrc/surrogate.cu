// surrogate.cu -- learned far field for the E/B update (no reference
// counterpart; it stands in for the far part of update_e_b_dynamic,
// IonSolver src/kernels/sim_kernels.cl:940-955).
//
// Split of the reference's sum over the depth-D LOD bins of one cell:
//   near : bins within Chebyshev distance R_NEAR (= 2) of the cell's own bin
//          (own bin excluded, as the reference excludes it) -- summed exactly
//          per cell (<= 124 terms instead of ~3511);
//   far  : all other bins in range -- smooth over one block, so it is taken
//          at the 8 corner cells of the cell's block and interpolated
//          trilinearly.  The 8 x 6 corner values of every block come from a
//          bias-free (linear) 3-D convolutional network on the LOD grid:
//          4 input channels (q, q vx, q vy, q vz per bin), 32 hidden
//          channels, 4 residual blocks of two 3^3 convolutions (dilations
//          (1,2) (2,4) (4,8) (1,1)), 48 output channels.  The target map is
//          linear in the sources, so the network is kept linear: scaling the
//          inputs scales the outputs exactly.
// Training runs on the GPU with the kernels below (FP32 forward, backward
// of data and weights, Adam); inference runs in BF16 on the tensor cores
// (mma.sync m16n8k16, FP32 accumulation).  Each step a sampled-cell check
// compares the surrogate against the exact sum on a few cells; above the
// tolerance the exact kernel recomputes the whole field.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include <cuda_bf16.h>

#include "field_kernels.cuh"
#include "ion_launch.h"
#include "surrogate.h"

namespace ion {

// ---------------------------------------------------------------------------
// geometry helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ int tap_off(int k, int a) { return (a == 0 ? k % 3 : a == 1 ? (k / 3) % 3 : k / 9) - 1; }

// ---------------------------------------------------------------------------
// exact far-field targets at the 8 corner cells of every block
//   src [4][V]: (q, qvx, qvy, qvz) per bin (bins below first_src are 0)
//   out [48][V]: channel = corner * 6 + component (Ex,Ey,Ez,Bx,By,Bz)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_far_targets(const float* src, int nd, float bs_x, float bs_y, float bs_z,
                                                     int rnear, float* out, int nsamples) {
    const int V = nd * nd * nd;
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)V * 8 * nsamples) return;
    const int s = (int)(gid / (V * 8));
    const int r = (int)(gid % (V * 8));
    const int v = r / 8, corner = r % 8;
    const int bx = v % nd, by = (v / nd) % nd, bz = v / (nd * nd);
    // corner cell coordinates (cells are at integer positions, bin centres at (i + 1/2) bs)
    const float px = bx * bs_x + ((corner & 1) ? bs_x - 1.0f : 0.0f);
    const float py = by * bs_y + ((corner & 2) ? bs_y - 1.0f : 0.0f);
    const float pz = bz * bs_z + ((corner & 4) ? bs_z - 1.0f : 0.0f);
    const float* S = src + (size_t)s * 4 * V;
    double e[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    for (int d = 0; d < V; d++) {
        const int dx = d % nd, dy = (d / nd) % nd, dz = d / (nd * nd);
        const int cheb = max(abs(dx - bx), max(abs(dy - by), abs(dz - bz)));
        if (cheb <= rnear) continue;
        const float q = S[d];
        const float qx = S[V + d], qy = S[2 * V + d], qz = S[3 * V + d];
        const double Rx = px - (dx + 0.5) * bs_x, Ry = py - (dy + 0.5) * bs_y, Rz = pz - (dz + 0.5) * bs_z;
        const double r2 = Rx * Rx + Ry * Ry + Rz * Rz;
        const double inv3 = 1.0 / (r2 * sqrt(r2));
        e[0] += q * Rx * inv3; e[1] += q * Ry * inv3; e[2] += q * Rz * inv3;
        b[0] += (qy * Rz - qz * Ry) * inv3; b[1] += (qz * Rx - qx * Rz) * inv3; b[2] += (qx * Ry - qy * Rx) * inv3;
    }
    float* O = out + (size_t)s * 48 * V;
    for (int c = 0; c < 3; c++) {
        O[(corner * 6 + c) * V + v] = (float)e[c];
        O[(corner * 6 + 3 + c) * V + v] = (float)b[c];
    }
}

// ---------------------------------------------------------------------------
// FP32 training kernels
// ---------------------------------------------------------------------------
constexpr int COG = 8;  // output channels per thread

// out[b][co][v] = (res ? res[b][co][v] : 0) + sum_ci sum_k w[co][ci][k] in[b][ci][v + dil*off_k]
__global__ void __launch_bounds__(128) k_conv_fwd(const float* in, const float* w, const float* res, float* out, int Cin,
                                                  int Cout, int dil, int nd, int B) {
    extern __shared__ float sw[];  // [COG][Cin][27]
    const int V = nd * nd * nd;
    const int co0 = blockIdx.y * COG;
    const int ncog = min(COG, Cout - co0);
    for (int i = threadIdx.x; i < ncog * Cin * 27; i += blockDim.x) sw[i] = w[(size_t)co0 * Cin * 27 + i];
    __syncthreads();
    const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long long)B * V) return;
    const int b = (int)(gid / V), v = (int)(gid % V);
    const int x = v % nd, y = (v / nd) % nd, z = v / (nd * nd);
    float acc[COG];
#pragma unroll
    for (int j = 0; j < COG; j++) acc[j] = 0.0f;
    const float* I = in + (size_t)b * Cin * V;
    for (int k = 0; k < 27; k++) {
        const int xx = x + dil * tap_off(k, 0), yy = y + dil * tap_off(k, 1), zz = z + dil * tap_off(k, 2);
        if (xx < 0 || yy < 0 || zz < 0 || xx >= nd || yy >= nd || zz >= nd) continue;
        const int nv = xx + (yy + zz * nd) * nd;
        for (int ci = 0; ci < Cin; ci++) {
            const float a = I[(size_t)ci * V + nv];
#pragma unroll
            for (int j = 0; j < COG; j++) acc[j] = fmaf(sw[(j * Cin + ci) * 27 + k], a, acc[j]);
        }
    }
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

__global__ void k_add(float* a, const float* b, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] += b[i];
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
// K = Cin*27, mma.sync.m16n8k16 (BF16 in, FP32 accumulate).
//   act [Cin][V] bf16 (one sample), wk [K][Cout] bf16 with k = tap*Cin + ci
//   out fp32 [Cout][V] (+ res), outb bf16 copy for the next layer
// One warp computes 16 voxels x all Cout (Cout / 8 n-tiles).
// ---------------------------------------------------------------------------
template <int NT>  // n-tiles of 8 output channels
__global__ void __launch_bounds__(128) k_conv_bf16(const __nv_bfloat16* act, const __nv_bfloat16* wk, const float* res,
                                                   float* out, __nv_bfloat16* outb, int Cin, int dil, int nd) {
    const int V = nd * nd * nd;
    const int Cout = NT * 8;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, tg = lane & 3;
    const int v0 = warp * 16;
    if (v0 >= V) return;
    float acc[NT][4];
#pragma unroll
    for (int t = 0; t < NT; t++) acc[t][0] = acc[t][1] = acc[t][2] = acc[t][3] = 0.0f;
    // voxel rows owned by this thread in the A fragment: v0 + g and v0 + g + 8
    const int va = v0 + g, vb = v0 + g + 8;
    const int xa = va % nd, ya = (va / nd) % nd, za = va / (nd * nd);
    const int xb = vb % nd, yb = (vb / nd) % nd, zb = vb / (nd * nd);
    const int K = Cin * 27;
    for (int k0 = 0; k0 < K; k0 += 16) {
        // A fragment: rows (va, vb), cols k0 + tg*2 + {0,1} and k0 + 8 + tg*2 + {0,1}
        uint32_t a[4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
#pragma unroll
            for (int rsel = 0; rsel < 2; rsel++) {
                __nv_bfloat16 pair[2];
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int kk = k0 + h * 8 + tg * 2 + e;
                    const int tap = kk / Cin, ci = kk % Cin;
                    const int x = (rsel ? xb : xa) + dil * tap_off(tap, 0);
                    const int y = (rsel ? yb : ya) + dil * tap_off(tap, 1);
                    const int z = (rsel ? zb : za) + dil * tap_off(tap, 2);
                    const bool in = kk < K && x >= 0 && y >= 0 && z >= 0 && x < nd && y < nd && z < nd;
                    pair[e] = in ? act[(size_t)ci * V + x + (y + z * nd) * nd] : __float2bfloat16(0.0f);
                }
                uint32_t u;
                memcpy(&u, pair, 4);
                a[h * 2 + rsel] = u;  // a0:(g,k lo) a1:(g+8,k lo) a2:(g,k hi) a3:(g+8,k hi)
            }
        }
#pragma unroll
        for (int t = 0; t < NT; t++) {
            // B fragment: k rows tg*2+{0,1} (+8), column n = t*8 + g
            __nv_bfloat16 b0[2], b1[2];
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int ka = k0 + tg * 2 + e, kb = k0 + 8 + tg * 2 + e;
                b0[e] = ka < K ? wk[(size_t)ka * Cout + t * 8 + g] : __float2bfloat16(0.0f);
                b1[e] = kb < K ? wk[(size_t)kb * Cout + t * 8 + g] : __float2bfloat16(0.0f);
            }
            uint32_t ub0, ub1;
            memcpy(&ub0, b0, 4);
            memcpy(&ub1, b1, 4);
            asm volatile(
                "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
                : "+f"(acc[t][0]), "+f"(acc[t][1]), "+f"(acc[t][2]), "+f"(acc[t][3])
                : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(ub0), "r"(ub1));
        }
    }
    // C fragment: (g, n = t*8 + tg*2 + {0,1}) and (g+8, same n)
#pragma unroll
    for (int t = 0; t < NT; t++) {
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int v = (e < 2) ? va : vb;
            const int n = t * 8 + tg * 2 + (e & 1);
            const size_t o = (size_t)n * V + v;
            const float val = acc[t][e] + (res ? res[o] : 0.0f);
            out[o] = val;
            if (outb) outb[o] = __float2bfloat16(val);
        }
    }
    (void)Cout;
}

__global__ void k_to_bf16(const float* x, __nv_bfloat16* y, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = __float2bfloat16(x[i]);
}

// wk[(tap*Cin + ci)][co] = w[co][ci][tap]
__global__ void k_pack_weights(const float* w, __nv_bfloat16* wk, int Cin, int Cout) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Cin * Cout * 27) return;
    const int co = i % Cout, kk = i / Cout, tap = kk / Cin, ci = kk % Cin;
    wk[i] = __float2bfloat16(w[((size_t)co * Cin + ci) * 27 + tap]);
}

// scales of the current sources: max |q| and max |q v| over the bins in range
__global__ void k_source_scale(const float* qu_lod, int V, int first, float* scales) {
    __shared__ float rq[256], rv[256];
    float mq = 0.0f, mv = 0.0f;
    for (int v = first + threadIdx.x; v < V; v += blockDim.x) {
        const float4 L = ((const float4*)qu_lod)[v];
        mq = fmaxf(mq, fabsf(L.x));
        mv = fmaxf(mv, fmaxf(fabsf(L.x * L.y), fmaxf(fabsf(L.x * L.z), fabsf(L.x * L.w))));
    }
    rq[threadIdx.x] = mq;
    rv[threadIdx.x] = mv;
    __syncthreads();
    for (int off = blockDim.x / 2; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            rq[threadIdx.x] = fmaxf(rq[threadIdx.x], rq[threadIdx.x + off]);
            rv[threadIdx.x] = fmaxf(rv[threadIdx.x], rv[threadIdx.x + off]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scales[0] = rq[0] > 0.0f ? rq[0] : 1.0f;
        scales[1] = rv[0] > 0.0f ? rv[0] : 1.0f;
    }
}

// ---------------------------------------------------------------------------
// per-cell field from the surrogate: exact near bins + interpolated far field
// Y [48][V] network output (normalised); scale: (sq*yE, sv*yB) from device
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_surrogate_cells(const DevLbm L, const float* Y, const float* scales, float yE,
                                                         float yB, int rnear) {
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= L.n || (L.flags[n] & F_BO) == F_S) return;
    uint32_t x, y, z;
    cell_xyz(L, n, x, y, z);
    const int nd = (int)L.nd, V = nd * nd * nd;
    const int bx = (int)(x / L.bsx), by = (int)(y / L.bsy), bz = (int)(z / L.bsz);
    const int own = bx + (by + bz * nd) * nd;
    const float fx = (float)x, fy = (float)y, fz = (float)z;
    float e[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    const float4* qu = (const float4*)L.qu_lod;
    for (int dz = max(bz - rnear, 0); dz <= min(bz + rnear, nd - 1); dz++)
        for (int dy = max(by - rnear, 0); dy <= min(by + rnear, nd - 1); dy++)
            for (int dx = max(bx - rnear, 0); dx <= min(bx + rnear, nd - 1); dx++) {
                const int d = dx + (dy + dz * nd) * nd;
                if (d == own || (uint32_t)d < L.first_src) continue;
                const float4 p = L.lod_pos[d], v = qu[d];
                add_src<true>(fx - p.x, fy - p.y, fz - p.z, make_float4(v.x, v.x * v.y, v.x * v.z, v.x * v.w), e, b);
            }
    // trilinear weights within the block (corner cells at offsets 0 and bs-1)
    const float tx = L.bsx > 1 ? (float)(x - bx * L.bsx) / (float)(L.bsx - 1) : 0.0f;
    const float ty = L.bsy > 1 ? (float)(y - by * L.bsy) / (float)(L.bsy - 1) : 0.0f;
    const float tz = L.bsz > 1 ? (float)(z - bz * L.bsz) / (float)(L.bsz - 1) : 0.0f;
    float far[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const float wgt = ((c & 1) ? tx : 1.0f - tx) * ((c & 2) ? ty : 1.0f - ty) * ((c & 4) ? tz : 1.0f - tz);
#pragma unroll
        for (int k = 0; k < 6; k++) far[k] = fmaf(wgt, Y[(size_t)(c * 6 + k) * V + own], far[k]);
    }
    const float sE = scales[0] * yE, sB = scales[1] * yB;
    const size_t N = L.n;
    L.e_dyn[n] = L.e_stat[n] + L.ke * (e[0] + sE * far[0]);
    L.e_dyn[N + n] = L.e_stat[N + n] + L.ke * (e[1] + sE * far[1]);
    L.e_dyn[2 * N + n] = L.e_stat[2 * N + n] + L.ke * (e[2] + sE * far[2]);
    L.b_dyn[n] = L.b_stat[n] + L.kmu * (b[0] + sB * far[3]);
    L.b_dyn[N + n] = L.b_stat[N + n] + L.kmu * (b[1] + sB * far[4]);
    L.b_dyn[2 * N + n] = L.b_stat[2 * N + n] + L.kmu * (b[2] + sB * far[5]);
}

// ---------------------------------------------------------------------------
// sampled exact check: exact dynamic E/B (FAST arithmetic, full bin range)
// on `count` cells picked by a hash of the step, compared with the values the
// surrogate wrote.  stats[0] = max |dE|, [1] = max |E|, [2] = max |dB|, [3] = max |B|
// (as float bits, atomicMax on non-negative floats)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

__global__ void __launch_bounds__(128) k_sample_check(const DevLbm L, uint32_t count, uint32_t salt, uint32_t* stats,
                                                     const unsigned long long* counters) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    salt += (uint32_t)counters[0] * 0x9e3779b9u;  // a new sample set every step, also under graph replay
    uint32_t n = hash32(i * 2654435761u + salt) % L.n;
    for (int tries = 0; tries < 8 && (L.flags[n] & F_BO) == F_S; tries++) n = hash32(n + 0x9e3779b9u) % L.n;
    if ((L.flags[n] & F_BO) == F_S) return;
    uint32_t x, y, z;
    cell_xyz(L, n, x, y, z);
    const uint32_t own = x / L.bsx + (y / L.bsy + z / L.bsz * L.nd) * L.nd;
    float e[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    const float4* qu = (const float4*)L.qu_lod;
    for (uint32_t d = L.first_src; d < L.n_lod_own; d++) {
        if (d == own) continue;
        const float4 p = L.lod_pos[d], v = qu[d];
        add_src<true>((float)x - p.x, (float)y - p.y, (float)z - p.z, make_float4(v.x, v.x * v.y, v.x * v.z, v.x * v.w),
                      e, b);
    }
    const size_t N = L.n;
    float dE = 0.0f, mE = 0.0f, dB = 0.0f, mB = 0.0f;
    for (int c = 0; c < 3; c++) {
        const float es = (L.e_dyn[c * N + n] - L.e_stat[c * N + n]) / L.ke;
        const float bs = (L.b_dyn[c * N + n] - L.b_stat[c * N + n]) / L.kmu;
        dE = fmaxf(dE, fabsf(es - e[c]));
        mE = fmaxf(mE, fabsf(e[c]));
        dB = fmaxf(dB, fabsf(bs - b[c]));
        mB = fmaxf(mB, fabsf(b[c]));
    }
    if (isnan(dE)) dE = 3.0e38f;
    if (isnan(dB)) dB = 3.0e38f;
    atomicMax(&stats[0], __float_as_uint(dE));
    atomicMax(&stats[1], __float_as_uint(mE));
    atomicMax(&stats[2], __float_as_uint(dB));
    atomicMax(&stats[3], __float_as_uint(mB));
}

// decides the fallback on the device: flag = 1 when a relative error exceeds tol
__global__ void k_sample_decide(uint32_t* stats, float tol, uint32_t* flag, float* last, unsigned long long* counters) {
    const float dE = __uint_as_float(stats[0]), mE = __uint_as_float(stats[1]);
    const float dB = __uint_as_float(stats[2]), mB = __uint_as_float(stats[3]);
    const float rE = mE > 0.0f ? dE / mE : dE, rB = mB > 0.0f ? dB / mB : dB;
    const bool bad = !(rE <= tol) || !(rB <= tol);
    *flag = bad ? 1u : 0u;
    last[0] = rE;
    last[1] = rB;
    counters[0] += 1ull;
    if (bad) counters[1] += 1ull;
    stats[0] = stats[1] = stats[2] = stats[3] = 0u;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {
struct LayerDef { int cin, cout, dil; };
const LayerDef kLayers[10] = {{4, 32, 1}, {32, 32, 1}, {32, 32, 2}, {32, 32, 2}, {32, 32, 4},
                              {32, 32, 4}, {32, 32, 8}, {32, 32, 1}, {32, 32, 1}, {32, 48, 1}};
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
    int rc = 0;
    rc |= alloc((void**)&w_, nw_ * 4);
    rc |= alloc((void**)&gw_, nw_ * 4);
    rc |= alloc((void**)&m_, nw_ * 4);
    rc |= alloc((void**)&v_, nw_ * 4);
    rc |= alloc((void**)&wt_, 32 * 48 * 27 * 4);
    rc |= alloc((void**)&wk_, nw_ * 2);
    rc |= alloc((void**)&scales_, 4 * 4);
    rc |= alloc((void**)&stats_, 8 * 4);
    rc |= alloc((void**)&flag_, 4);
    rc |= alloc((void**)&last_, 2 * 4);
    rc |= alloc((void**)&counters_, 2 * 8);
    rc |= alloc((void**)&xin_, (size_t)4 * V_ * 4);
    rc |= alloc((void**)&yout_, (size_t)48 * V_ * 4);
    rc |= alloc((void**)&ha_, (size_t)32 * V_ * 4);
    rc |= alloc((void**)&hb_, (size_t)32 * V_ * 4);
    rc |= alloc((void**)&ab_, (size_t)32 * V_ * 2);
    rc |= alloc((void**)&bb_, (size_t)32 * V_ * 2);
    if (rc) return ION_E_NOMEM;
    // He-style initialisation scaled down so the residual stack starts near identity
    std::mt19937 gen(12345);
    std::vector<float> w(nw_);
    for (int l = 0; l < 10; l++) {
        const float sd = (l >= 1 && l <= 8 ? 0.1f : 1.0f) / std::sqrt((float)kLayers[l].cin * 27.0f);
        std::normal_distribution<float> nd1(0.0f, sd);
        for (size_t i = 0; i < (size_t)kLayers[l].cin * kLayers[l].cout * 27; i++) w[woff_[l] + i] = nd1(gen);
    }
    cudaMemcpy(w_, w.data(), nw_ * 4, cudaMemcpyHostToDevice);
    ready_ = false;
    return cudaGetLastError() == cudaSuccess ? ION_OK : ION_E_CUDA;
}

// FP32 forward of a batch; acts: 9 activation buffers [B][32][V] + output [B][48][V]
void Surrogate::forward_fp32(const float* X, int B, std::vector<float*>& acts, float* Y, cudaStream_t s) {
    auto conv = [&](const float* in, int l, const float* res, float* out) {
        const LayerDef& d = kLayers[l];
        dim3 grid(blocks_for((size_t)B * V_, 128), (d.cout + COG - 1) / COG);
        k_conv_fwd<<<grid, 128, COG * d.cin * 27 * 4, s>>>(in, w_ + woff_[l], res, out, d.cin, d.cout, d.dil, nd_, B);
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
        k_conv_fwd<<<grid, 128, COG * d.cout * 27 * 4, s>>>(gout, wt_, res, gin, d.cout, d.cin, d.dil, nd_, B);
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

int Surrogate::train(int nsamples, int epochs, int batch, float lr, uint64_t seed, cudaStream_t s, float* rel_err) {
    // training snapshots: random charge and current per bin, exact far-field targets
    const size_t xs = (size_t)4 * V_, ys = (size_t)48 * V_;
    float *X = nullptr, *T = nullptr;
    if (cudaMalloc(&X, xs * nsamples * 4) != cudaSuccess || cudaMalloc(&T, ys * nsamples * 4) != cudaSuccess) {
        cudaFree(X);
        cudaGetLastError();
        return ION_E_NOMEM;
    }
    {
        std::mt19937_64 gen(seed);
        std::uniform_real_distribution<float> U(-1.0f, 1.0f);
        std::vector<float> h(xs * nsamples);
        for (int sidx = 0; sidx < nsamples; sidx++)
            for (int c = 0; c < 4; c++)
                for (int v = 0; v < V_; v++) h[sidx * xs + c * V_ + v] = v >= first_ ? U(gen) : 0.0f;
        cudaMemcpy(X, h.data(), h.size() * 4, cudaMemcpyHostToDevice);
    }
    k_far_targets<<<blocks_for((size_t)V_ * 8 * nsamples, 256), 256, 0, s>>>(X, nd_, bs_[0], bs_[1], bs_[2], RNEAR, T,
                                                                              nsamples);
    // normalisation of the E and B channel groups
    std::vector<float> th(ys * std::min(nsamples, 64));
    cudaMemcpyAsync(th.data(), T, th.size() * 4, cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    double se = 0, sb = 0;
    size_t ne = 0, nb = 0;
    for (size_t i = 0; i < th.size(); i++) {
        const int ch = (int)((i / V_) % 48) % 6;
        if (ch < 3) { se += (double)th[i] * th[i]; ne++; } else { sb += (double)th[i] * th[i]; nb++; }
    }
    yE_ = (float)std::sqrt(se / std::max<size_t>(ne, 1));
    yB_ = (float)std::sqrt(sb / std::max<size_t>(nb, 1));
    if (!(yE_ > 0)) yE_ = 1.0f;
    if (!(yB_ > 0)) yB_ = 1.0f;
    {
        std::vector<float> scale(48 * (size_t)V_);
        for (int ch = 0; ch < 48; ch++)
            for (int v = 0; v < V_; v++) scale[(size_t)ch * V_ + v] = 1.0f / (ch % 6 < 3 ? yE_ : yB_);
        float* d_scale = nullptr;
        cudaMalloc(&d_scale, scale.size() * 4);
        cudaMemcpy(d_scale, scale.data(), scale.size() * 4, cudaMemcpyHostToDevice);
        // T *= scale per sample (elementwise with the per-sample pattern)
        std::vector<float> all(ys * nsamples);
        cudaMemcpy(all.data(), T, all.size() * 4, cudaMemcpyDeviceToHost);
        for (int sidx = 0; sidx < nsamples; sidx++)
            for (size_t i = 0; i < ys; i++) all[sidx * ys + i] *= scale[i];
        cudaMemcpy(T, all.data(), all.size() * 4, cudaMemcpyHostToDevice);
        cudaFree(d_scale);
    }
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
    for (int ep = 0; ep < epochs && !rc; ep++) {
        const float lr_ep = lr * (ep < epochs / 2 ? 1.0f : ep < 3 * epochs / 4 ? 0.3f : 0.1f);
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
        loss_.push_back((float)(ep_loss / std::max(nb_, 1)));
        if (cudaGetLastError() != cudaSuccess) rc = ION_E_CUDA;
    }
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
        k_pack_weights<<<blocks_for((size_t)d.cin * d.cout * 27, 256), 256, 0, s>>>(w_ + woff_[l], wk_ + woff_[l], d.cin,
                                                                                    d.cout);
    }
}

// BF16 tensor-core forward of one sample X [4][V] (fp32) -> yout_ [48][V]
void Surrogate::infer_bf16(const float* X, cudaStream_t s) {
    // residual stream h in fp32 (ha_/hb_), bf16 copies for the next conv (ab_/bb_)
    k_to_bf16<<<blocks_for((size_t)4 * V_, 256), 256, 0, s>>>(X, bb_, (size_t)4 * V_);
    const unsigned grid = blocks_for((size_t)(V_ / 16) * 32, 128);
    auto conv = [&](const __nv_bfloat16* in, int l, const float* res, float* out, __nv_bfloat16* outb) {
        const LayerDef& d = kLayers[l];
        if (d.cout == 32) k_conv_bf16<4><<<grid, 128, 0, s>>>(in, wk_ + woff_[l], res, out, outb, d.cin, d.dil, nd_);
        else k_conv_bf16<6><<<grid, 128, 0, s>>>(in, wk_ + woff_[l], res, out, outb, d.cin, d.dil, nd_);
    };
    conv(bb_, 0, nullptr, ha_, ab_);  // h0
    for (int i = 0; i < 4; i++) {
        conv(ab_, 1 + 2 * i, nullptr, hb_, bb_);  // t_i (fp32 copy unused)
        conv(bb_, 2 + 2 * i, ha_, ha_, ab_);      // h_{i+1} = h_i + conv(t_i)
    }
    conv(ab_, 9, nullptr, yout_, nullptr);
}

void Surrogate::step(const DevLbm& L, cudaStream_t s, uint32_t salt) {
    k_source_scale<<<1, 256, 0, s>>>(L.qu_lod, V_, first_, scales_);
    k_pack_input_dev(L, s);
    infer_bf16(xin_, s);
    k_surrogate_cells<<<blocks_for(L.n, 256), 256, 0, s>>>(L, yout_, scales_, yE_, yB_, RNEAR);
    k_sample_check<<<blocks_for(check_cells_, 128), 128, 0, s>>>(L, check_cells_, salt, stats_, counters_);
    k_sample_decide<<<1, 1, 0, s>>>(stats_, tol_, flag_, last_, counters_);
}

// network input from the LOD table: X[c][v] = (q, q vx, q vy, q vz) divided by
// the step's source scales; bins below first_src are no sources (sim_kernels.cl:943)
__global__ void k_pack_input_scaled(const float* qu_lod, int V, int first, const float* scales, float* X) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V) return;
    const float4 L = ((const float4*)qu_lod)[v];
    const bool use = v >= first;
    const float sq = scales[0], sv = scales[1];
    X[v] = use ? L.x / sq : 0.0f;
    X[V + v] = use ? L.x * L.y / sv : 0.0f;
    X[2 * V + v] = use ? L.x * L.z / sv : 0.0f;
    X[3 * V + v] = use ? L.x * L.w / sv : 0.0f;
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
    const size_t xs = (size_t)4 * V_, ys = (size_t)48 * V_;
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
        if (cudaStreamSynchronize(s) != cudaSuccess) rc = ION_E_CUDA;
    }
    for (auto p : acts) cudaFree(p);
    for (auto p : g) cudaFree(p);
    cudaFree(X); cudaFree(T); cudaFree(Y); cudaFree(gY); cudaFree(loss);
    cudaGetLastError();
    return rc;
}

int Surrogate::forward(const float* hX, float* hY, bool bf16, cudaStream_t s) {
    const size_t xs = (size_t)4 * V_, ys = (size_t)48 * V_;
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
        if (cudaStreamSynchronize(s) != cudaSuccess) rc = ION_E_CUDA;
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
    const uint32_t hdr[4] = {0x474f5253u /* "SROG" */, 1u, (uint32_t)nd_, (uint32_t)nw_};
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
    bool ok = fread(hdr, 4, 4, f) == 4 && hdr[0] == 0x474f5253u && hdr[1] == 1u && hdr[2] == (uint32_t)nd_ &&
              hdr[3] == (uint32_t)nw_ && fread(&yE_, 4, 1, f) == 1 && fread(&yB_, 4, 1, f) == 1 &&
              fread(w.data(), 4, nw_, f) == nw_;
    fclose(f);
    if (!ok) return ION_E_FORMAT;
    if (cudaMemcpy(w_, w.data(), nw_ * 4, cudaMemcpyHostToDevice) != cudaSuccess) return ION_E_CUDA;
    pack_bf16(s);
    ready_ = true;
    return ION_OK;
}

}  // namespace ion
