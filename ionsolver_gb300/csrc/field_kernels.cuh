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

// n / d by a multiply-high: floor(n m / 2^32) with m = floor((2^32 - 1) / d) + 1 (d > 1).
// With n = q d + r, n m / 2^32 = n / d + n e / 2^32 with 0 <= e < 1, and n e / 2^32 < 1 / d
// whenever n d < 2^32, so the floor is q (division by invariant integers, Granlund &
// Montgomery 1994).  Callers keep n d < 2^32.
struct Magic {
    uint32_t d, m;
    __device__ explicit Magic(uint32_t dd) : d(dd), m(dd > 1u ? 0xFFFFFFFFu / dd + 1u : 0u) {}
    __device__ __forceinline__ uint32_t div(uint32_t n) const { return d > 1u ? __umulhi(n, m) : n; }
};

// LOD bins of one domain, one thread block per bin: warps 1..7 stream the
// bin's cells (ascending cell index) through shared memory in slabs of
// LB_SLAB cells, double-buffered, while lanes 0..3 of warp 0 add charge and
// the three velocity components one cell after another -- the same sequence
// of float additions as lod_bin_warp.  A cell outside the fluid is stored as
// -0.0f, which leaves every float (+0 included) unchanged under
// round-to-nearest addition, so the sums need no branch and the summing
// lanes read four cells per shared-memory load.

constexpr uint32_t LB_THREADS = 256, LB_SLAB = 512;
struct LodSmem {
    float v[2][4][LB_SLAB];  // [buffer][component][cell]
};

static __global__ void __launch_bounds__(LB_THREADS) k_lod_bins(const DevLbm L) {
    __shared__ __align__(16) LodSmem sm;
    const uint32_t bin = blockIdx.x;
    if (bin >= L.n_bins) {  // bins of the lower LOD levels stay zero (single domain)
        if (threadIdx.x < 4u) L.qu_lod[(size_t)bin * 4u + threadIdx.x] = 0.0f;
        return;
    }
    const uint32_t nd = L.nd;
    const uint32_t bx = bin % nd, by = (bin / nd) % nd, bz = bin / (nd * nd);
    const uint32_t cells = L.bsx * L.bsy * L.bsz;
    const uint32_t nslabs = (cells + LB_SLAB - 1u) / LB_SLAB;
    const size_t N = L.n;
    const Magic mx(L.bsx), mxy(L.bsx * L.bsy);
    const bool magic = (uint64_t)cells * (L.bsx * L.bsy) < (1ull << 32);  // Magic's bound (bins of <= ~2^16 cells)
    auto load = [&](uint32_t k) {  // warps 1..7; the slab is padded with -0.0f to a multiple of 4 cells
        const uint32_t base = k * LB_SLAB;
        const uint32_t cnt = min(LB_SLAB, cells - base);
        const uint32_t padded = (cnt + 3u) & ~3u;
        float(*v)[LB_SLAB] = sm.v[k & 1u];
#pragma unroll 3
        for (uint32_t i = threadIdx.x - 32u; i < padded; i += LB_THREADS - 32u) {
            float4 c = make_float4(-0.0f, -0.0f, -0.0f, -0.0f);
            if (i < cnt) {  // all five loads in flight at once; the flag selects afterwards
                const uint32_t li = base + i;
                uint32_t lx, ly, lz;
                if (magic) {
                    lz = mxy.div(li);
                    const uint32_t r = li - lz * mxy.d;
                    ly = mx.div(r);
                    lx = r - ly * mx.d;
                } else {
                    lx = li % L.bsx; ly = (li / L.bsx) % L.bsy; lz = li / (L.bsx * L.bsy);
                }
                const uint32_t n = (bx * L.bsx + lx) + ((by * L.bsy + ly) + (bz * L.bsz + lz) * L.ny) * L.nx;
                const uint8_t f = L.flags[n];
                const float4 a = make_float4(L.q[n], L.lod_cell[n], L.lod_cell[N + n], L.lod_cell[2 * N + n]);
                if ((f & F_BO) != F_S) c = a;
            }
            v[0][i] = c.x; v[1][i] = c.y; v[2][i] = c.z; v[3][i] = c.w;
        }
    };
    if (threadIdx.x >= 32u) load(0);
    __syncthreads();
    float acc = 0.0f;
    for (uint32_t k = 0; k < nslabs; k++) {
        if (threadIdx.x >= 32u) {
            if (k + 1u < nslabs) load(k + 1u);
        } else if (threadIdx.x < 4u) {
            const uint32_t quads = (min(LB_SLAB, cells - k * LB_SLAB) + 3u) / 4u;
            const float4* v = (const float4*)sm.v[k & 1u][threadIdx.x];
            uint32_t i = 0;
            for (; i + 4u <= quads; i += 4u) {  // 16 cells: loads first, then the dependent additions
                const float4 a = v[i], b = v[i + 1u], c = v[i + 2u], d = v[i + 3u];
                acc = acc + a.x; acc = acc + a.y; acc = acc + a.z; acc = acc + a.w;
                acc = acc + b.x; acc = acc + b.y; acc = acc + b.z; acc = acc + b.w;
                acc = acc + c.x; acc = acc + c.y; acc = acc + c.z; acc = acc + c.w;
                acc = acc + d.x; acc = acc + d.y; acc = acc + d.z; acc = acc + d.w;
            }
            for (; i < quads; i++) {
                const float4 a = v[i];
                acc = acc + a.x; acc = acc + a.y; acc = acc + a.z; acc = acc + a.w;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x < 4u) L.qu_lod[(size_t)bin * 4u + threadIdx.x] = acc;
}

// ---------------------------------------------------------------------------
// bulk asynchronous copy global -> shared, completion counted on an mbarrier
// (PTX ISA: cp.async.bulk, mbarrier.*; sm_90 and later)
// ---------------------------------------------------------------------------
constexpr uint32_t SRC_CHUNK = 256;  // sources per shared-memory tile

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
        const float y = __frcp_rn(c3);  // the three IEEE divides by c3, via one reciprocal
        const float px = div_rn_shared(rx, c3, y), py = div_rn_shared(ry, c3, y), pz = div_rn_shared(rz, c3, y);
        e[0] = e[0] + val.x * px; e[1] = e[1] + val.x * py; e[2] = e[2] + val.x * pz;
        const float bx = val.z * pz - val.w * py, by = val.w * px - val.y * pz, bz = val.y * py - val.z * px;
        b[0] = b[0] + val.x * bx; b[1] = b[1] + val.x * by; b[2] = b[2] + val.x * bz;
    }
}

// FAST far field in coordinates relative to an origin o near the cells (the
// centre of their brick): with c' = c - o and p' = p - o,
//   |R|^2 = (|c'|^2 + |p'|^2) - 2 c'.p'                 (4 operations, no R,
//         summed as (c'z mz + (c'x mx + |c'|^2)) + (c'y my + |p'|^2), m = -2 p':
//         two independent chains, one dependent step fewer before the rsqrt)
//   E = sum q R/|R|^3 = c' S - P,   S = sum q/|R|^3,  P = sum q p'/|R|^3
//   B = sum qv x R/|R|^3 = A x c' - W,  A = sum qv/|R|^3,  W = sum (qv x p')/|R|^3
// so one source costs 16 operations; |c'| is at most ~11 cells, which keeps
// the expansion of |R|^2 and the split sums free of cancellation at the
// distances that occur (the own bin is excluded).
// One source, pre-broadcast into pairs for far_fast2 (m = -2 p'):
// (mx,mx,my,my) (mz,mz,pp,pp) (q,q,qpx,qpx) (qpy,qpy,qpz,qpz) (qvx,qvx,qvy,qvy) (qvz,qvz,wx,wx) (wy,wy,wz,wz)
struct FastSrc {
    float4 d[7];
};

// A source of the brick's near box (summed directly, see eb_tile) enters the far sums
// as q = 0 at p' = 0 with |p'|^2 = 1: |R|^2 = |c'|^2 + 1 >= 1 stays finite, so it
// adds exactly zero (the cell's own bin, possibly at |R| = 0, is one of them).
__device__ __forceinline__ void fast_src(FastSrc& f, float4 p, float4 v, float ox, float oy, float oz, bool in_box) {
    // p = bin centre, v = (q, vx, vy, vz)
    if (in_box) { p = make_float4(ox, oy, oz, 0.0f); v = make_float4(0.0f, 0.0f, 0.0f, 0.0f); }
    const float px = p.x - ox, py = p.y - oy, pz = p.z - oz;
    const float pp = in_box ? 1.0f : fmaf(pz, pz, fmaf(py, py, px * px));
    const float q = v.x;
    const float qx = q * v.y, qy = q * v.z, qz = q * v.w;
    const float wx = qy * pz - qz * py, wy = qz * px - qx * pz, wz = qx * py - qy * px;
    const float mx = -2.0f * px, my = -2.0f * py, mz = -2.0f * pz;
    const float qpx = q * px, qpy = q * py, qpz = q * pz;
    f.d[0] = make_float4(mx, mx, my, my);
    f.d[1] = make_float4(mz, mz, pp, pp);
    f.d[2] = make_float4(q, q, qpx, qpx);
    f.d[3] = make_float4(qpy, qpy, qpz, qpz);
    f.d[4] = make_float4(qx, qx, qy, qy);
    f.d[5] = make_float4(qz, qz, wx, wx);
    f.d[6] = make_float4(wy, wy, wz, wz);
}

// Far-field sums of two cells (the two halves of every pair).
struct Pair3 {
    P2 x, y, z;
};
struct FarSums {  // per cell pair: S, P, A, W
    P2 S;
    Pair3 P, A, W;
};
__device__ __forceinline__ void far_zero(FarSums& f) {
    f.S = 0ull;
    f.P = {0ull, 0ull, 0ull};
    f.A = f.P;
    f.W = f.P;
}
__device__ __forceinline__ void far_fast2(const Pair3& c, P2 cc, const FastSrc& src, FarSums& f) {
    const ulonglong2* u = reinterpret_cast<const ulonglong2*>(src.d);
    const ulonglong2 d0 = u[0], d1 = u[1], d2 = u[2], d3 = u[3], d4 = u[4], d5 = u[5], d6 = u[6];
    const P2 ra = fma2(c.z, d1.x, fma2(c.x, d0.x, cc)), rb = fma2(c.y, d0.y, d1.y);
    const P2 r2 = add2(ra, rb);
    float i0, i1;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(i0) : "f"(lo32(r2)));
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(i1) : "f"(hi32(r2)));
    const P2 inv = pk(i0, i1);
    const P2 inv3 = mul2(mul2(inv, inv), inv);
    f.S = fma2(d2.x, inv3, f.S);
    f.P.x = fma2(d2.y, inv3, f.P.x);
    f.P.y = fma2(d3.x, inv3, f.P.y);
    f.P.z = fma2(d3.y, inv3, f.P.z);
    f.A.x = fma2(d4.x, inv3, f.A.x);
    f.A.y = fma2(d4.y, inv3, f.A.y);
    f.A.z = fma2(d5.x, inv3, f.A.z);
    f.W.x = fma2(d5.y, inv3, f.W.x);
    f.W.y = fma2(d6.x, inv3, f.W.y);
    f.W.z = fma2(d6.y, inv3, f.W.z);
}

// far_fast2 for one half (hi = false: first cell, true: second) -- the same
// operations in the same order, for the source chunk that holds a cell's own bin
__device__ __forceinline__ void far_fast1(const Pair3& c, P2 cc, const FastSrc& S, FarSums& f, bool hi) {
    const float4 d0 = S.d[0], d1 = S.d[1], d2 = S.d[2], d3 = S.d[3], d4 = S.d[4], d5 = S.d[5], d6 = S.d[6];
    const float ra = fmaf(half(c.z, hi), d1.x, fmaf(half(c.x, hi), d0.x, half(cc, hi))), rb = fmaf(half(c.y, hi), d0.z, d1.z);
    const float r2 = ra + rb;
    float inv;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(inv) : "f"(r2));
    const float inv3 = (inv * inv) * inv;
    set_half(f.S, hi, fmaf(d2.x, inv3, half(f.S, hi)));
    set_half(f.P.x, hi, fmaf(d2.z, inv3, half(f.P.x, hi)));
    set_half(f.P.y, hi, fmaf(d3.x, inv3, half(f.P.y, hi)));
    set_half(f.P.z, hi, fmaf(d3.z, inv3, half(f.P.z, hi)));
    set_half(f.A.x, hi, fmaf(d4.x, inv3, half(f.A.x, hi)));
    set_half(f.A.y, hi, fmaf(d4.z, inv3, half(f.A.y, hi)));
    set_half(f.A.z, hi, fmaf(d5.x, inv3, half(f.A.z, hi)));
    set_half(f.W.x, hi, fmaf(d5.z, inv3, half(f.W.x, hi)));
    set_half(f.W.y, hi, fmaf(d6.x, inv3, half(f.W.y, hi)));
    set_half(f.W.z, hi, fmaf(d6.z, inv3, half(f.W.z, hi)));
}

// E and B of one half from its far sums (relative coordinates c')
__device__ __forceinline__ void far_finish(const Pair3& c, const FarSums& f, bool hi, float* e, float* b) {
    const float cx = half(c.x, hi), cy = half(c.y, hi), cz = half(c.z, hi);
    const float S = half(f.S, hi);
    const float Px = half(f.P.x, hi), Py = half(f.P.y, hi), Pz = half(f.P.z, hi);
    const float Ax = half(f.A.x, hi), Ay = half(f.A.y, hi), Az = half(f.A.z, hi);
    const float Wx = half(f.W.x, hi), Wy = half(f.W.y, hi), Wz = half(f.W.z, hi);
    e[0] = e[0] + (cx * S - Px);
    e[1] = e[1] + (cy * S - Py);
    e[2] = e[2] + (cz * S - Pz);
    b[0] = b[0] + ((Ay * cz - Az * cy) - Wx);
    b[1] = b[1] + ((Az * cx - Ax * cz) - Wy);
    b[2] = b[2] + ((Ax * cy - Ay * cx) - Wz);
}

// One source of the near box for a cell pair, directly: R = c - p per lane (exact),
// q R/|R|^3 and (q v x R)/|R|^3 added to the pair's sums.  A lane that must skip the
// source (its own bin, or an inactive cell) gets |R|^2 = 1 and weight 0, so it adds
// exact zeros.
__device__ __forceinline__ void near_pair(P2 rx, P2 ry, P2 rz, float4 v, bool use_lo, bool use_hi, Pair3& e,
                                          Pair3& b) {
    const P2 r2 = fma2(rz, rz, fma2(ry, ry, mul2(rx, rx)));
    float i0, i1;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(i0) : "f"(use_lo ? lo32(r2) : 1.0f));
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(i1) : "f"(use_hi ? hi32(r2) : 1.0f));
    const P2 inv = pk(i0, i1);
    const P2 w = mul2(mul2(mul2(inv, inv), inv), pk(use_lo ? 1.0f : 0.0f, use_hi ? 1.0f : 0.0f));
    const P2 s = mul2(pk(v.x, v.x), w);
    e.x = fma2(s, rx, e.x);
    e.y = fma2(s, ry, e.y);
    e.z = fma2(s, rz, e.z);
    const P2 qx = pk(v.y, v.y), qy = pk(v.z, v.z), qz = pk(v.w, v.w);
    const P2 cx = fma2(qy, rz, mul2(pk(-v.w, -v.w), ry));
    const P2 cy = fma2(qz, rx, mul2(pk(-v.y, -v.y), rz));
    const P2 cz = fma2(qx, ry, mul2(pk(-v.z, -v.z), rx));
    b.x = fma2(w, cx, b.x);
    b.y = fma2(w, cy, b.y);
    b.z = fma2(w, cz, b.z);
}
constexpr uint32_t NEAR_BATCH = 256;  // near-box bins staged at a time (2 float4 each, within sm.fast)

// Shared-memory staging area of one thread block; the mbarrier phase of each
// buffer is tracked in `uses` so one block can process many tiles.
template <bool FAST>
struct EbSmem {
    float4 pos[2][SRC_CHUNK];          // bin centres, as copied
    float4 val[2][SRC_CHUNK];          // (q, vx, vy, vz), as copied
    FastSrc fast[FAST ? SRC_CHUNK : 1];  // FAST: the chunk being summed, in pairs
    uint64_t bar[2];
};

template <class SM>
__device__ __forceinline__ void eb_init(SM& sm) {
    if (threadIdx.x == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
}


// Near field of one cell: its aligned block of near_x*near_y*near_z cells
// (sim_kernels.cl:907-938), skipping the cell itself and uncharged cells.
template <bool FAST>
__device__ __forceinline__ void near_field(const DevLbm& L, uint32_t n, uint32_t x, uint32_t y, uint32_t z, float* e,
                                           float* b) {
    const size_t N = L.n;
    const uint32_t x0 = (x / L.near_x) * L.near_x, y0 = (y / L.near_y) * L.near_y, z0 = (z / L.near_z) * L.near_z;
    const uint32_t x1 = min(x0 + L.near_x, L.nx), y1 = min(y0 + L.near_y, L.ny), z1 = min(z0 + L.near_z, L.nz);
    for (uint32_t cx = x0; cx < x1; cx++)
        for (uint32_t cy = y0; cy < y1; cy++)
            for (uint32_t cz = z0; cz < z1; cz++) {
                const uint32_t nc = cx + (cy + cz * L.ny) * L.nx;
                if (nc == n) continue;
                const float qc = L.q[nc];
                if (qc == 0.0f) continue;
                const float vx = L.u[nc], vy = L.u[N + nc], vz = L.u[2 * N + nc];
                const float4 val = FAST ? make_float4(qc, qc * vx, qc * vy, qc * vz) : make_float4(qc, vx, vy, vz);
                add_src<FAST>((float)x - (float)cx, (float)y - (float)cy, (float)z - (float)cz, val, e, b);
            }
}

// One past the last source bin summed.  The reference reads bins [n_lod_own - 8^D,
// n_lod_own), but its bin sums only write indices below 8^D and clear_qu_lod
// (sim_kernels.cl:995-1003) zeroes the rest every step, so the trailing n_lod_own - 8^D
// terms are q = 0 times a finite factor (those bins lie outside the box): +-0.  Adding
// +-0 changes no sum here -- a sum starts at +0 and, under round-to-nearest, can only
// become +0 again by cancellation, never -0 -- so both modes stop at 8^D and BITWISE
// stays bit-identical (14% fewer terms at every depth).
template <bool FAST>
__device__ __forceinline__ uint32_t src_last(const DevLbm& L) { return min(L.n_lod_own, L.n_bins); }

// Issues the bulk copies of source chunk c into buffer c & 1 (one thread).
template <class SM>
__device__ __forceinline__ void eb_issue(const DevLbm& L, SM& sm, uint32_t c, uint32_t last) {
    const uint32_t first = L.first_src;
    const uint32_t base = first + c * SRC_CHUNK;
    const uint32_t cnt = min(SRC_CHUNK, last - base);
    const uint32_t buf = c & 1u;
    mbar_expect_tx(&sm.bar[buf], 2u * cnt * 16u);
    bulk_g2s(&sm.pos[buf][0], L.lod_pos + base, cnt * 16u, &sm.bar[buf]);
    bulk_g2s(&sm.val[buf][0], (const float4*)L.qu_lod + base, cnt * 16u, &sm.bar[buf]);
}

__device__ __forceinline__ void eb_store(const DevLbm& L, uint32_t n, const float* e, const float* b) {
    const size_t N = L.n;
    L.e_dyn[n] = L.e_stat[n] + L.ke * e[0];
    L.e_dyn[N + n] = L.e_stat[N + n] + L.ke * e[1];
    L.e_dyn[2 * N + n] = L.e_stat[2 * N + n] + L.ke * e[2];
    L.b_dyn[n] = L.b_stat[n] + L.kmu * b[0];
    L.b_dyn[N + n] = L.b_stat[N + n] + L.kmu * b[1];
    L.b_dyn[2 * N + n] = L.b_stat[2 * N + n] + L.kmu * b[2];
}

// E/B of the cells of one brick (or, with 128 threads, of half of one:
// sub = 0, 1) of domain L.  Returns false (block-uniform) when a staged tile
// did not arrive within its wait limit.  Per cell the sources are added in
// the reference's order; the cell's own bin is skipped by a check that runs
// only in the one source chunk that can contain it.  FAST holds the cells in
// pairs (2j, 2j+1) and advances both with packed FP32 instructions.
template <bool FAST>
__device__ __forceinline__ bool eb_tile(const DevLbm& L, const uint32_t brick, const uint32_t sub, EbSmem<FAST>& sm,
                                        uint32_t (&uses)[2]) {
    static_assert(EB_CPT % 2 == 0, "cells are processed in pairs");
    constexpr uint32_t NP = EB_CPT / 2;
    const uint32_t nbx = (L.nx + EB_BX - 1) / EB_BX, nby = (L.ny + EB_BY - 1) / EB_BY;
    const uint32_t bx = brick % nbx, by = (brick / nbx) % nby, bz = brick / (nbx * nby);
    const uint32_t x = bx * EB_BX + threadIdx.x % EB_BX;
    const uint32_t y = by * EB_BY + threadIdx.x / EB_BX + sub * (blockDim.x / EB_BX);
    // brick centre: the origin of the FAST coordinates
    const float ox = (float)(bx * EB_BX) + 0.5f * (float)(EB_BX - 1);
    const float oy = (float)(by * EB_BY) + 0.5f * (float)(EB_BY - 1);
    const float oz = (float)(bz * EB_CPT) + 0.5f * (float)(EB_CPT - 1);
    // depth-D LOD bins [first_src, n_lod_own) except the cell's own (sim_kernels.cl:940-955);
    // the first chunk's copy starts now, so it lands while the near field is summed
    const uint32_t first = L.first_src, last = src_last<FAST>(L);
    const uint32_t nchunks = (last - first + SRC_CHUNK - 1u) / SRC_CHUNK;
    if (threadIdx.x == 0 && nchunks > 0) eb_issue(L, sm, 0, last);
    float e[EB_CPT][3], b[EB_CPT][3];  // near field (and, BITWISE, everything)
    float ax[EB_CPT], ay[EB_CPT], az[EB_CPT];  // BITWISE: absolute coordinates
    float rx[EB_CPT], ry[EB_CPT], rz[EB_CPT];  // FAST: coordinates relative to the brick centre
    FarSums fs[NP];
    uint32_t own[EB_CPT];
    bool active[EB_CPT];
#pragma unroll
    for (uint32_t k = 0; k < EB_CPT; k++) {
        const uint32_t z = bz * EB_CPT + k;
        const bool inside = x < L.nx && y < L.ny && z < L.nz;
        const uint32_t n = inside ? x + (y + z * L.ny) * L.nx : 0u;
        active[k] = inside && (L.flags[n] & F_BO) != F_S;
        own[k] = active[k] ? x / L.bsx + (y / L.bsy + z / L.bsz * L.nd) * L.nd : 0xFFFFFFFFu;
        ax[k] = (float)x; ay[k] = (float)y; az[k] = (float)z;
        rx[k] = (float)x - ox; ry[k] = (float)y - oy; rz[k] = (float)z - oz;
#pragma unroll
        for (int c = 0; c < 3; c++) { e[k][c] = 0.0f; b[k][c] = 0.0f; }
        if (active[k]) near_field<FAST>(L, n, x, y, z, e[k], b[k]);
    }
    // FAST: the bins within one bin (Chebyshev) of the brick's cells -- its near box --
    // are summed directly, q R/|R|^3 with R = c - p exact (cell and bin coordinates are
    // integers and halves), each cell skipping its own bin.  For such a close source the
    // far sums' split E = c' S - P (below) cancels, which costs up to 10x the rounding
    // error of the direct form; the far loop sees these bins with q = 0 (fast_src).
    uint32_t box_lo[3] = {0u, 0u, 0u}, box_hi[3] = {0u, 0u, 0u};
    if constexpr (FAST) {
        // the whole brick's box, also for a half-brick block: every cell then sums the
        // same sources directly, whatever the block shape (batches pick 128 or 256)
        const uint32_t lo[3] = {bx * EB_BX, by * EB_BY, bz * EB_CPT};
        const uint32_t hi[3] = {min(lo[0] + EB_BX, L.nx) - 1u, min(lo[1] + EB_BY, L.ny) - 1u, min(lo[2] + EB_CPT, L.nz) - 1u};
        const uint32_t bsz[3] = {L.bsx ? L.bsx : 1u, L.bsy ? L.bsy : 1u, L.bsz ? L.bsz : 1u};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const uint32_t b0 = lo[a] / bsz[a], b1 = hi[a] / bsz[a];
            box_lo[a] = b0 > 0u ? b0 - 1u : 0u;
            box_hi[a] = min(b1 + 1u, L.nd - 1u);
        }
        // The box's bins are staged in shared memory (sm.fast is free until the far loop)
        // in batches of NEAR_BATCH; every thread then sums them for its cells, the pair
        // (2j, 2j+1) -- the same x and y, z one apart -- in packed instructions.
        const uint32_t ex = box_hi[0] - box_lo[0] + 1u, ey = box_hi[1] - box_lo[1] + 1u;
        const uint32_t nbox = ex * ey * (box_hi[2] - box_lo[2] + 1u);
        float4* stage = reinterpret_cast<float4*>(sm.fast);  // [NEAR_BATCH] centres + index, then (q, q v)
        Pair3 en[NP], bn[NP];
#pragma unroll
        for (uint32_t j = 0; j < NP; j++) { en[j] = {0ull, 0ull, 0ull}; bn[j] = en[j]; }
        const P2 px2 = pk(ax[0], ax[0]), py2 = pk(ay[0], ay[0]);
        for (uint32_t b0 = 0; b0 < nbox; b0 += NEAR_BATCH) {
            const uint32_t cnt = min(NEAR_BATCH, nbox - b0);
            __syncthreads();  // the previous batch is consumed
            for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) {
                const uint32_t t = b0 + i;
                const uint32_t d = (box_lo[0] + t % ex) + ((box_lo[1] + (t / ex) % ey) + (box_lo[2] + t / (ex * ey)) * L.nd) * L.nd;
                const float4 pd = L.lod_pos[d], v = reinterpret_cast<const float4*>(L.qu_lod)[d];
                const bool src = d >= first && d < last;  // inside the reference's source range
                stage[i] = make_float4(pd.x, pd.y, pd.z, __uint_as_float(d));
                stage[NEAR_BATCH + i] = src ? make_float4(v.x, v.x * v.y, v.x * v.z, v.x * v.w) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            __syncthreads();
            for (uint32_t i = 0; i < cnt; i++) {
                const float4 pd = stage[i], v = stage[NEAR_BATCH + i];
                const uint32_t d = __float_as_uint(pd.w);
                const P2 rx = add2(px2, pk(-pd.x, -pd.x)), ry = add2(py2, pk(-pd.y, -pd.y));
#pragma unroll
                for (uint32_t j = 0; j < NP; j++)
                    near_pair(rx, ry, pk(az[2 * j] - pd.z, az[2 * j + 1] - pd.z), v,
                              active[2 * j] && d != own[2 * j], active[2 * j + 1] && d != own[2 * j + 1], en[j], bn[j]);
            }
        }
        __syncthreads();  // sm.fast is written by the far loop next
#pragma unroll
        for (uint32_t j = 0; j < NP; j++)
#pragma unroll
            for (uint32_t h = 0; h < 2; h++) {
                float* ek = e[2 * j + h];
                float* bk = b[2 * j + h];
                ek[0] = ek[0] + half(en[j].x, h); ek[1] = ek[1] + half(en[j].y, h); ek[2] = ek[2] + half(en[j].z, h);
                bk[0] = bk[0] + half(bn[j].x, h); bk[1] = bk[1] + half(bn[j].y, h); bk[2] = bk[2] + half(bn[j].z, h);
            }
    }
    Pair3 cp[NP];  // FAST: the relative coordinates in pairs, and |c'|^2
    P2 cc[NP];
#pragma unroll
    for (uint32_t j = 0; j < NP; j++) {
        cp[j] = {pk(rx[2 * j], rx[2 * j + 1]), pk(ry[2 * j], ry[2 * j + 1]), pk(rz[2 * j], rz[2 * j + 1])};
        cc[j] = pk(fmaf(rz[2 * j], rz[2 * j], fmaf(ry[2 * j], ry[2 * j], rx[2 * j] * rx[2 * j])),
                   fmaf(rz[2 * j + 1], rz[2 * j + 1], fmaf(ry[2 * j + 1], ry[2 * j + 1], rx[2 * j + 1] * rx[2 * j + 1])));
        far_zero(fs[j]);
    }

    bool ok = true;
    uint32_t c = 0;
    for (; c < nchunks; c++) {
        const uint32_t buf = c & 1u;
        if (threadIdx.x == 0 && c + 1 < nchunks) eb_issue(L, sm, c + 1, last);
        const bool landed = mbar_wait(&sm.bar[buf], uses[buf] & 1u, L.wait_limit);
        ok = __syncthreads_and(landed) != 0;  // block-uniform
        if (!ok) break;
        uses[buf]++;
        const uint32_t base = first + c * SRC_CHUNK;
        const uint32_t cnt = min(SRC_CHUNK, last - base);
        bool here = false;
#pragma unroll
        for (uint32_t k = 0; k < EB_CPT; k++) here |= (own[k] - base) < cnt;
        const bool any_own = __any_sync(0xFFFFFFFFu, here);  // this chunk holds some cell's own bin
        if constexpr (FAST) {
            for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x)
            {
                const uint32_t d = base + k, dx = d % L.nd, dy = (d / L.nd) % L.nd, dz = d / (L.nd * L.nd);
                const bool in_box = dx >= box_lo[0] && dx <= box_hi[0] && dy >= box_lo[1] && dy <= box_hi[1] &&
                                    dz >= box_lo[2] && dz <= box_hi[2];
                fast_src(sm.fast[k], sm.pos[buf][k], sm.val[buf][k], ox, oy, oz, in_box);
            }
            __syncthreads();
            const FastSrc* src = sm.fast;
            if (any_own) {
                for (uint32_t s = 0; s < cnt; s++) {
                    const FastSrc S = src[s];
#pragma unroll
                    for (uint32_t j = 0; j < NP; j++) {
                        const bool lo_ok = base + s != own[2 * j], hi_ok = base + s != own[2 * j + 1];
                        if (lo_ok && hi_ok) {
                            far_fast2(cp[j], cc[j], S, fs[j]);
                        } else {  // one of the pair is in its own bin: scalar steps on the other
                            if (lo_ok) far_fast1(cp[j], cc[j], S, fs[j], false);
                            if (hi_ok) far_fast1(cp[j], cc[j], S, fs[j], true);
                        }
                    }
                }
            } else {
#pragma unroll 1
                for (uint32_t s = 0; s < cnt; s++) {
                    const FastSrc S = src[s];
#pragma unroll
                    for (uint32_t j = 0; j < NP; j++) far_fast2(cp[j], cc[j], S, fs[j]);
                }
            }
        } else {
            const float4* sp = &sm.pos[buf][0];
            const float4* sv = &sm.val[buf][0];
            if (any_own) {
                for (uint32_t s = 0; s < cnt; s++) {
                    const float4 p = sp[s], v = sv[s];
#pragma unroll
                    for (uint32_t k = 0; k < EB_CPT; k++)
                        if (base + s != own[k]) add_src<false>(ax[k] - p.x, ay[k] - p.y, az[k] - p.z, v, e[k], b[k]);
                }
            } else {
#pragma unroll 2
                for (uint32_t s = 0; s < cnt; s++) {
                    const float4 p = sp[s], v = sv[s];
#pragma unroll
                    for (uint32_t k = 0; k < EB_CPT; k++) add_src<false>(ax[k] - p.x, ay[k] - p.y, az[k] - p.z, v, e[k], b[k]);
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
        if (!active[k]) continue;
        if constexpr (FAST) far_finish(cp[k / 2], fs[k / 2], (k & 1u) != 0, e[k], b[k]);
        eb_store(L, x + (y + (bz * EB_CPT + k) * L.ny) * L.nx, e[k], b[k]);
    }
    return true;
}

// The exact update, run only when *gate != 0 (the surrogate's fallback decision)
static __global__ void __launch_bounds__(256, 2) k_update_e_b_gated(const DevLbm L, uint32_t* err, const uint32_t* gate) {
    if (*gate == 0u) return;
    __shared__ __align__(16) EbSmem<true> sm;
    eb_init(sm);
    uint32_t uses[2] = {0u, 0u};
    if (!eb_tile<true>(L, blockIdx.x, 0u, sm, uses) && threadIdx.x == 0) atomicExch(err, 1u);
}

// FAST: 2 blocks of 256 threads per SM (registers); BITWISE: 3
static __global__ void __launch_bounds__(256, 2) k_update_e_b_fast(const DevLbm L, uint32_t* err) {
    __shared__ __align__(16) EbSmem<true> sm;
    eb_init(sm);
    uint32_t uses[2] = {0u, 0u};
    if (!eb_tile<true>(L, blockIdx.x, 0u, sm, uses) && threadIdx.x == 0) atomicExch(err, 1u);
}
static __global__ void __launch_bounds__(256, 3) k_update_e_b_exact(const DevLbm L, uint32_t* err) {
    __shared__ __align__(16) EbSmem<false> sm;
    eb_init(sm);
    uint32_t uses[2] = {0u, 0u};
    if (!eb_tile<false>(L, blockIdx.x, 0u, sm, uses) && threadIdx.x == 0) atomicExch(err, 1u);
}

}  // namespace ion
