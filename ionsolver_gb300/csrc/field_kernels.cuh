// field_kernels.cuh -- LOD bin sums and the dynamic E/B field update
// (IonSolver src/kernels/sim_kernels.cl:666-677, 897-1003) on sm_103a.
//
// LOD bins.  The reference accumulates every fluid cell's charge and
// velocity/volume into its depth-D bin with float atomics.  Here one warp
// owns one bin: lanes fetch 32 cells at a time in ascending cell order and
// lanes 0..3 (charge, ux, uy, uz) add them one after another.  The result
// is the sum the reference produces when its work-items run in index order,
// and it is the same on every run.
//
// E/B update.  Every fluid cell sums q R/|R|^3 (Coulomb) and
// q v x R/|R|^3 (Biot-Savart) over its near-field block and over the depth-D
// LOD bins [n_lod_own - 8^D, n_lod_own) except its own bin.  A thread block
// stages the bin table (centre + charge + velocity) through shared memory
// with bulk asynchronous copies (cp.async.bulk, completion on an mbarrier),
// double-buffered, and every thread walks the sources in ascending order.
//   BITWISE: the reference's operations and order (IEEE sqrt and divides).
//   FAST:    one reciprocal square root per source, charge-weighted velocity
//            precomputed per source, FMA contraction.
#pragma once
#include "ion_device.cuh"
#include "ion_launch.h"

namespace ion {

// ---------------------------------------------------------------------------
// LOD bins: one warp per bin (bins >= 8^D are cleared, as clear_qu_lod does)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void lod_bin_warp(const DevLbm& L, const uint32_t bin, const uint32_t lane) {
    float acc = 0.0f;
    if (bin < L.n_bins) {
        const uint32_t nd = L.nd;
        const uint32_t bx = bin % nd, by = (bin / nd) % nd, bz = bin / (nd * nd);
        const uint32_t cells = L.bsx * L.bsy * L.bsz;
        const size_t N = L.n;
        for (uint32_t base = 0; base < cells; base += 32u) {
            const uint32_t li = base + lane;
            float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f, v3 = 0.0f;
            bool has = false;
            if (li < cells) {
                const uint32_t lx = li % L.bsx, ly = (li / L.bsx) % L.bsy, lz = li / (L.bsx * L.bsy);
                const uint32_t n = (bx * L.bsx + lx) + ((by * L.bsy + ly) + (bz * L.bsz + lz) * L.ny) * L.nx;
                has = (L.flags[n] & F_BO) != F_S;
                if (has) { v0 = L.q[n]; v1 = L.lod_cell[n]; v2 = L.lod_cell[N + n]; v3 = L.lod_cell[2 * N + n]; }
            }
            const uint32_t cnt = cells - base < 32u ? cells - base : 32u;
            for (uint32_t k = 0; k < cnt; k++) {
                const float a0 = __shfl_sync(0xFFFFFFFFu, v0, k);
                const float a1 = __shfl_sync(0xFFFFFFFFu, v1, k);
                const float a2 = __shfl_sync(0xFFFFFFFFu, v2, k);
                const float a3 = __shfl_sync(0xFFFFFFFFu, v3, k);
                const int hk = __shfl_sync(0xFFFFFFFFu, (int)has, k);
                if (hk) {
                    const float a = lane == 0u ? a0 : lane == 1u ? a1 : lane == 2u ? a2 : a3;
                    acc = acc + a;
                }
            }
        }
    }
    if (lane < 4u) L.qu_lod[(size_t)bin * 4u + lane] = acc;
}

static __global__ void __launch_bounds__(256) k_lod_bins(const DevLbm L) {
    const uint32_t bin = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (bin < L.n_lod_own) lod_bin_warp(L, bin, threadIdx.x & 31u);
}

// ---------------------------------------------------------------------------
// bulk asynchronous copy global -> shared, completion counted on an mbarrier
// (PTX ISA: cp.async.bulk, mbarrier.*; sm_90 and later)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}
// Waits for the phase with the given parity; gives up after `limit` polls
// and returns false (the caller records the failure and skips the tile).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

constexpr uint32_t SRC_CHUNK = 256;  // sources per shared-memory tile
constexpr uint32_t WAIT_LIMIT = 1u << 24;

template <bool FAST>
__device__ __forceinline__ void add_src(float rx, float ry, float rz, float4 val, float* e, float* b) {
    if constexpr (FAST) {
        // val = (q, q*vx, q*vy, q*vz)
        const float r2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
        float inv;  // PTX rsqrt.approx (one MUFU op; r2 >= 1/4 here, so FTZ never applies)
        asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(r2));
        const float inv3 = inv * inv * inv;
        const float s = val.x * inv3;
        e[0] = fmaf(s, rx, e[0]); e[1] = fmaf(s, ry, e[1]); e[2] = fmaf(s, rz, e[2]);
        const float cx = fmaf(val.z, rz, -val.w * ry), cy = fmaf(val.w, rx, -val.y * rz), cz = fmaf(val.y, ry, -val.z * rx);
        b[0] = fmaf(inv3, cx, b[0]); b[1] = fmaf(inv3, cy, b[1]); b[2] = fmaf(inv3, cz, b[2]);
    } else {
        // val = (q, vx, vy, vz); sim_kernels.cl:931-935 / 950-954
        const float s = sqrtf((rx * rx + ry * ry) + rz * rz);
        const float c3 = (s * s) * s;
        const float px = rx / c3, py = ry / c3, pz = rz / c3;
        e[0] = e[0] + val.x * px; e[1] = e[1] + val.x * py; e[2] = e[2] + val.x * pz;
        const float bx = val.z * pz - val.w * py, by = val.w * px - val.y * pz, bz = val.y * py - val.z * px;
        b[0] = b[0] + val.x * bx; b[1] = b[1] + val.x * by; b[2] = b[2] + val.x * bz;
    }
}

// FAST far field of one source: E += q R/|R|^3 and, for B, the two sums
// A += qv/|R|^3 and W += (qv x p)/|R|^3, from which B = A x c - W at the end
// (qv x (c - p) = qv x c - qv x p): 3 FMA per source instead of 9.
// p = (px, py, pz, q), qv = (q vx, q vy, q vz, -), w = qv x p.
__device__ __forceinline__ void far_fast(float cx, float cy, float cz, float4 p, float4 qv, float4 w, float* e, float* A,
                                         float* W) {
    const float rx = cx - p.x, ry = cy - p.y, rz = cz - p.z;
    const float r2 = fmaf(rz, rz, fmaf(ry, ry, rx * rx));
    float inv;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(r2));
    const float inv3 = inv * inv * inv;
    const float s = p.w * inv3;
    e[0] = fmaf(s, rx, e[0]); e[1] = fmaf(s, ry, e[1]); e[2] = fmaf(s, rz, e[2]);
    A[0] = fmaf(inv3, qv.x, A[0]); A[1] = fmaf(inv3, qv.y, A[1]); A[2] = fmaf(inv3, qv.z, A[2]);
    W[0] = fmaf(inv3, w.x, W[0]); W[1] = fmaf(inv3, w.y, W[1]); W[2] = fmaf(inv3, w.z, W[2]);
}

// Shared-memory staging area of one thread block; the mbarrier phase of each
// buffer is tracked in `uses` so one block can process many tiles.
struct EbSmem {
    float4 pos[2][SRC_CHUNK];
    float4 val[2][SRC_CHUNK];
    float4 wv[2][SRC_CHUNK];  // FAST: qv x p of each source
    uint64_t bar[2];
};

__device__ __forceinline__ void eb_init(EbSmem& sm) {
    if (threadIdx.x == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
}


// E/B of the cells [tile, tile + EB_CPT*blockDim.x) of domain L.  Returns
// false (block-uniform) when a staged tile did not arrive within its wait
// limit.  Per cell the sources are added in the reference's order; the
// cell's own bin is skipped by a check that runs only in the one source
// chunk that can contain it.
template <bool FAST>
__device__ __forceinline__ bool eb_tile(const DevLbm& L, const uint32_t tile, EbSmem& sm, uint32_t (&uses)[2]) {
    const uint32_t N = L.n;
    float fx[EB_CPT], fy[EB_CPT], fz[EB_CPT], e[EB_CPT][3], b[EB_CPT][3];
    float Af[EB_CPT][3], Wf[EB_CPT][3];  // FAST far-field sums of the split cross product
    uint32_t own[EB_CPT];
    bool active[EB_CPT];
#pragma unroll
    for (uint32_t k = 0; k < EB_CPT; k++) {
        const uint32_t n = tile + threadIdx.x + k * blockDim.x;
        active[k] = n < N && (L.flags[n] & F_BO) != F_S;
        uint32_t x = 0, y = 0, z = 0;
        if (n < N) cell_xyz(L, n, x, y, z);
        fx[k] = (float)x; fy[k] = (float)y; fz[k] = (float)z;
        own[k] = n < N ? x / L.bsx + (y / L.bsy + z / L.bsz * L.nd) * L.nd : 0xFFFFFFFFu;
        if (!active[k]) own[k] = 0xFFFFFFFFu;
#pragma unroll
        for (int c = 0; c < 3; c++) { e[k][c] = 0.0f; b[k][c] = 0.0f; Af[k][c] = 0.0f; Wf[k][c] = 0.0f; }
        // near field: the cell's aligned block (sim_kernels.cl:907-938)
        if (active[k]) {
            const uint32_t x0 = (x / L.near_x) * L.near_x, y0 = (y / L.near_y) * L.near_y, z0 = (z / L.near_z) * L.near_z;
            const uint32_t x1 = min(x0 + L.near_x, L.nx), y1 = min(y0 + L.near_y, L.ny), z1 = min(z0 + L.near_z, L.nz);
            for (uint32_t cx = x0; cx < x1; cx++)
                for (uint32_t cy = y0; cy < y1; cy++)
                    for (uint32_t cz = z0; cz < z1; cz++) {
                        const uint32_t nc = cx + (cy + cz * L.ny) * L.nx;
                        if (nc == n) continue;
                        const float qc = L.q[nc];
                        if (qc == 0.0f) continue;
                        const float vx = L.u[nc], vy = L.u[(size_t)N + nc], vz = L.u[2 * (size_t)N + nc];
                        const float4 val = FAST ? make_float4(qc, qc * vx, qc * vy, qc * vz) : make_float4(qc, vx, vy, vz);
                        add_src<FAST>(fx[k] - (float)cx, fy[k] - (float)cy, fz[k] - (float)cz, val, e[k], b[k]);
                    }
        }
    }

    // depth-D LOD bins [first_src, n_lod_own) except the cell's own (sim_kernels.cl:940-955)
    const uint32_t first = L.first_src, last = L.n_lod_own;
    const uint32_t nchunks = (last - first + SRC_CHUNK - 1u) / SRC_CHUNK;
    const float4* qu = (const float4*)L.qu_lod;
    auto issue = [&](uint32_t c) {
        const uint32_t base = first + c * SRC_CHUNK;
        const uint32_t cnt = min(SRC_CHUNK, last - base);
        const uint32_t buf = c & 1u;
        mbar_expect_tx(&sm.bar[buf], 2u * cnt * 16u);
        bulk_g2s(&sm.pos[buf][0], L.lod_pos + base, cnt * 16u, &sm.bar[buf]);
        bulk_g2s(&sm.val[buf][0], qu + base, cnt * 16u, &sm.bar[buf]);
    };
    if (threadIdx.x == 0 && nchunks > 0) issue(0);
    bool ok = true;
    uint32_t c = 0;
    for (; c < nchunks; c++) {
        const uint32_t buf = c & 1u;
        if (threadIdx.x == 0 && c + 1 < nchunks) issue(c + 1);
        const bool landed = mbar_wait(&sm.bar[buf], uses[buf] & 1u, WAIT_LIMIT);
        ok = __syncthreads_and(landed) != 0;  // block-uniform
        if (!ok) break;
        uses[buf]++;
        const uint32_t base = first + c * SRC_CHUNK;
        const uint32_t cnt = min(SRC_CHUNK, last - base);
        if constexpr (FAST) {  // per source: (p, q), q v and q v x p, once per tile
            for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
                const float4 p = sm.pos[buf][k], v = sm.val[buf][k];
                const float qx = v.x * v.y, qy = v.x * v.z, qz = v.x * v.w;
                sm.pos[buf][k] = make_float4(p.x, p.y, p.z, v.x);
                sm.val[buf][k] = make_float4(qx, qy, qz, 0.0f);
                sm.wv[buf][k] = make_float4(qy * p.z - qz * p.y, qz * p.x - qx * p.z, qx * p.y - qy * p.x, 0.0f);
            }
            __syncthreads();
        }
        bool here = false;
#pragma unroll
        for (uint32_t k = 0; k < EB_CPT; k++) here |= (own[k] - base) < cnt;
        const float4* sp = &sm.pos[buf][0];
        const float4* sv = &sm.val[buf][0];
        const float4* sw = &sm.wv[buf][0];
        if (__any_sync(0xFFFFFFFFu, here)) {  // this chunk holds some cell's own bin
            for (uint32_t s = 0; s < cnt; s++) {
                const float4 p = sp[s], v = sv[s];
                if constexpr (FAST) {
                    const float4 w = sw[s];
#pragma unroll
                    for (uint32_t k = 0; k < EB_CPT; k++)
                        if (base + s != own[k]) far_fast(fx[k], fy[k], fz[k], p, v, w, e[k], Af[k], Wf[k]);
                } else {
#pragma unroll
                    for (uint32_t k = 0; k < EB_CPT; k++)
                        if (base + s != own[k]) add_src<false>(fx[k] - p.x, fy[k] - p.y, fz[k] - p.z, v, e[k], b[k]);
                }
            }
        } else {
#pragma unroll 2
            for (uint32_t s = 0; s < cnt; s++) {
                const float4 p = sp[s], v = sv[s];
                if constexpr (FAST) {
                    const float4 w = sw[s];
#pragma unroll
                    for (uint32_t k = 0; k < EB_CPT; k++) far_fast(fx[k], fy[k], fz[k], p, v, w, e[k], Af[k], Wf[k]);
                } else {
#pragma unroll
                    for (uint32_t k = 0; k < EB_CPT; k++)
                        add_src<false>(fx[k] - p.x, fy[k] - p.y, fz[k] - p.z, v, e[k], b[k]);
                }
            }
        }
        __syncthreads();  // everyone is done with this buffer before it is refilled
    }
    if (!ok) {
        // a tile did not arrive in time: wait (bounded) for the copies still in
        // flight and leave the outputs untouched
        if (threadIdx.x == 0)
            for (uint32_t k = c; k < nchunks && k <= c + 1u; k++) mbar_wait(&sm.bar[k & 1u], uses[k & 1u] & 1u, WAIT_LIMIT);
        return false;
    }
#pragma unroll
    for (uint32_t k = 0; k < EB_CPT; k++) {
        const uint32_t n = tile + threadIdx.x + k * blockDim.x;
        if (!active[k]) continue;
        if constexpr (FAST) {  // B = near part + A x c - W
            b[k][0] = b[k][0] + ((Af[k][1] * fz[k] - Af[k][2] * fy[k]) - Wf[k][0]);
            b[k][1] = b[k][1] + ((Af[k][2] * fx[k] - Af[k][0] * fz[k]) - Wf[k][1]);
            b[k][2] = b[k][2] + ((Af[k][0] * fy[k] - Af[k][1] * fx[k]) - Wf[k][2]);
        }
        L.e_dyn[n] = L.e_stat[n] + L.ke * e[k][0];
        L.e_dyn[(size_t)N + n] = L.e_stat[(size_t)N + n] + L.ke * e[k][1];
        L.e_dyn[2 * (size_t)N + n] = L.e_stat[2 * (size_t)N + n] + L.ke * e[k][2];
        L.b_dyn[n] = L.b_stat[n] + L.kmu * b[k][0];
        L.b_dyn[(size_t)N + n] = L.b_stat[(size_t)N + n] + L.kmu * b[k][1];
        L.b_dyn[2 * (size_t)N + n] = L.b_stat[2 * (size_t)N + n] + L.kmu * b[k][2];
    }
    return true;
}

// The exact update, run only when *gate != 0 (the surrogate's fallback decision)
static __global__ void __launch_bounds__(256) k_update_e_b_gated(const DevLbm L, uint32_t* err, const uint32_t* gate) {
    if (*gate == 0u) return;
    __shared__ __align__(16) EbSmem sm;
    eb_init(sm);
    uint32_t uses[2] = {0u, 0u};
    if (!eb_tile<true>(L, blockIdx.x * blockDim.x * EB_CPT, sm, uses) && threadIdx.x == 0) atomicExch(err, 1u);
}

template <bool FAST>
static __global__ void __launch_bounds__(256) k_update_e_b(const DevLbm L, uint32_t* err) {
    __shared__ __align__(16) EbSmem sm;
    eb_init(sm);
    uint32_t uses[2] = {0u, 0u};
    if (!eb_tile<FAST>(L, blockIdx.x * blockDim.x * EB_CPT, sm, uses) && threadIdx.x == 0) atomicExch(err, 1u);
}

}  // namespace ion
