// setup_kernels.cu -- geometry and static-field kernels, FP64 reductions.
//
//   voxelize  : IonSolver src/kernels/sim_kernels.cl:1150-1231 (one thread
//               per bounding-box column, Moeller-Trumbore in both ray
//               directions, 16-bit hit distances, parity with correction).
//   psi / B   : sim_kernels.cl:1234-1276.  The reference loops over all N
//               cells for each of the (N+2)^3 potential points and tests the
//               magnet flag; here the magnet cells are first compacted into an
//               ascending index list (same summation order, ~N/N_magnet less
//               work) and staged through shared memory.
//   static E  : sim_kernels.cl:1278-1300, same compaction over charged cells.
//   FP64 sums : deterministic two-pass tree reductions of decoded DDFs.
#include "ion_device.cuh"
#include "ion_launch.h"
#include "reduce_f64.cuh"

namespace ion {

// ---------------------------------------------------------------------------
// voxelisation
// ---------------------------------------------------------------------------
struct V3 { float x, y, z; };
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 vcross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ float vdot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ int iclamp(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

__global__ void __launch_bounds__(128) k_voxelize(const DevLbm L, VoxArgs A) {
    const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A.columns) return;
    const int nx = (int)L.nx, ny = (int)L.ny, nz = (int)L.nz;
    const int dir = A.direction;
    uint32_t c[3];
    if (dir == 0) { c[0] = (uint32_t)iclamp((int)A.x0, 0, nx - 1); c[1] = a % L.ny; c[2] = a / L.ny; }
    else if (dir == 1) { c[0] = a / L.nz; c[1] = (uint32_t)iclamp((int)A.y0, 0, ny - 1); c[2] = a % L.nz; }
    else { c[0] = a % L.nx; c[1] = a / L.nx; c[2] = (uint32_t)iclamp((int)A.z0, 0, nz - 1); }
    const V3 org = {(((float)c[0] + 0.5f) - 0.5f * (float)nx) + (0.5f * (float)nx - 0.5f),
                    (((float)c[1] + 0.5f) - 0.5f * (float)ny) + (0.5f * (float)ny - 0.5f),
                    (((float)c[2] + 0.5f) - 0.5f * (float)nz) + (0.5f * (float)nz - 0.5f)};
    bool outside;
    if (dir == 0) outside = org.y < A.y0 || org.z < A.z0 || org.y >= A.y1 || org.z >= A.z1;
    else if (dir == 1) outside = org.x < A.x0 || org.z < A.z0 || org.x >= A.x1 || org.z >= A.z1;
    else outside = org.x < A.x0 || org.y < A.y0 || org.x >= A.x1 || org.y >= A.y1;
    if (outside) return;
    const V3 rdir = {(float)(dir == 0), (float)(dir == 1), (float)(dir == 2)};
    uint16_t dist[64];
    for (int i = 0; i < 64; i++) dist[i] = 0;
    uint32_t hits = 0, back = 0;
    for (uint32_t i = 0; i < A.ntri; i++) {
        const V3 P0 = {A.p0[3 * i], A.p0[3 * i + 1], A.p0[3 * i + 2]};
        const V3 P1 = {A.p1[3 * i], A.p1[3 * i + 1], A.p1[3 * i + 2]};
        const V3 P2 = {A.p2[3 * i], A.p2[3 * i + 1], A.p2[3 * i + 2]};
        const V3 e1 = vsub(P1, P0), e2 = vsub(P2, P0), s0 = vsub(org, P0);
        const V3 pv = vcross(rdir, e2), qv = vcross(s0, e1);
        const float inv = 1.0f / vdot(e1, pv);
        const float su = inv * vdot(s0, pv), sv = inv * vdot(rdir, qv), sd = inv * vdot(e2, qv);
        if (su >= 0.0f && su < 1.0f && sv >= 0.0f && su + sv < 1.0f) {
            if (sd > 0.0f) {
                if (hits < 64u && sd < 65536.0f) dist[hits] = (uint16_t)sd;
                hits++;
            } else {
                back++;
            }
        }
    }
    const uint32_t ns = hits < 64u ? hits : 64u;
    for (uint32_t i = 1; i < ns; i++) {
        const uint16_t key = dist[i];
        int k = (int)i - 1;
        while (k >= 0 && dist[k] > key) { dist[k + 1] = dist[k]; k--; }
        dist[k + 1] = key;
    }
    bool inside = (hits % 2u) && (back % 2u);
    uint32_t next = (hits % 2u) != (back % 2u);
    const uint32_t h0 = c[dir];
    const uint32_t hmax = dir == 0 ? (uint32_t)iclamp((int)A.x1, 0, nx) : dir == 1 ? (uint32_t)iclamp((int)A.y1, 0, ny)
                                                                                  : (uint32_t)iclamp((int)A.z1, 0, nz);
    const uint32_t last = hits - 1u < 63u ? hits - 1u : 63u;
    const uint32_t hmesh = h0 + (uint32_t)dist[last];
    const size_t N = L.n;
    for (uint32_t hh = h0; hh < hmax; hh++) {
        while (next < hits && hh > h0 + (uint32_t)dist[next < 63u ? next : 63u]) { inside = !inside; next++; }
        inside = inside && (next < hits && hh < hmesh);
        uint32_t cc[3] = {c[0], c[1], c[2]};
        cc[dir] = hh;
        const uint32_t n = cc[0] + (cc[1] + cc[2] * L.ny) * L.nx;
        if (inside) {
            L.flags[n] = (uint8_t)((L.flags[n] & ~F_BO) | A.flag);
            if (L.ext_mhd) {
                if (A.flag & F_M) { L.b_dyn[n] = A.mx; L.b_dyn[N + n] = A.my; L.b_dyn[2 * N + n] = A.mz; }
                else if ((A.flag & F_F) || (A.flag & F_C)) L.b_dyn[n] = A.mx;
            }
        }
    }
}

void launch_voxelize(const DevLbm& L, const VoxArgs& A, cudaStream_t s) {
    k_voxelize<<<grid_for(A.columns, 128), 128, 0, s>>>(L, A);
}

// ---------------------------------------------------------------------------
// order-preserving compaction of cells whose flags match a mask
// (count per 1024-cell tile -> exclusive scan of tile counts -> scatter)
// ---------------------------------------------------------------------------
constexpr uint32_t CT = 1024;

__global__ void __launch_bounds__(CT) k_compact_count(const uint8_t* flags, uint32_t n, uint8_t mask, uint32_t* tiles) {
    const uint32_t i = blockIdx.x * CT + threadIdx.x;
    const int hit = i < n && (flags[i] & mask) != 0;
    const int c = __syncthreads_count(hit);
    if (threadIdx.x == 0) tiles[blockIdx.x] = (uint32_t)c;
}

__global__ void __launch_bounds__(CT) k_compact_scan(uint32_t* tiles, uint32_t ntiles, uint32_t* total) {
    __shared__ uint32_t part[CT];
    const uint32_t per = (ntiles + CT - 1) / CT;
    const uint32_t b = threadIdx.x * per, e = min(b + per, ntiles);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; i++) s += tiles[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = 1; off < CT; off <<= 1) {  // inclusive Hillis-Steele scan
        const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = threadIdx.x ? part[threadIdx.x - 1] : 0u;
    for (uint32_t i = b; i < e; i++) { const uint32_t c = tiles[i]; tiles[i] = run; run += c; }
    if (threadIdx.x == CT - 1) *total = part[CT - 1];
}

__global__ void __launch_bounds__(CT) k_compact_scatter(const uint8_t* flags, uint32_t n, uint8_t mask,
                                                        const uint32_t* tiles, uint32_t* out) {
    __shared__ uint32_t warp_count[CT / 32];
    const uint32_t i = blockIdx.x * CT + threadIdx.x;
    const bool hit = i < n && (flags[i] & mask) != 0;
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t ball = __ballot_sync(0xFFFFFFFFu, hit);
    if (lane == 0) warp_count[wid] = __popc(ball);
    __syncthreads();
    uint32_t off = tiles[blockIdx.x];
    for (uint32_t w = 0; w < wid; w++) off += warp_count[w];
    if (hit) out[off + __popc(ball & ((1u << lane) - 1u))] = i;
}

void launch_compact(const DevLbm& L, uint8_t mask, uint32_t* tiles, uint32_t* list, uint32_t* total, cudaStream_t s) {
    const uint32_t ntiles = (L.n + CT - 1) / CT;
    k_compact_count<<<ntiles, CT, 0, s>>>(L.flags, L.n, mask, tiles);
    k_compact_scan<<<1, CT, 0, s>>>(tiles, ntiles, total);
    k_compact_scatter<<<ntiles, CT, 0, s>>>(L.flags, L.n, mask, tiles, list);
}

// ---------------------------------------------------------------------------
// magnetic scalar potential on the padded grid, stored in E_dyn
// ---------------------------------------------------------------------------
constexpr uint32_t MAG_TILE = 256;

__global__ void __launch_bounds__(256) k_psi(const DevLbm L, const uint32_t* mags, const uint32_t* count, float* psi) {
    __shared__ float4 s_p[MAG_TILE];  // (x+1, y+1, z+1) as float
    __shared__ float4 s_m[MAG_TILE];  // magnetisation
    const uint32_t l0 = L.nx + 2, l1 = L.ny + 2;
    const uint32_t np = (l0 * l1) * (L.nz + 2);
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t t = i % (l0 * l1);
    const float cx = (float)(t % l0), cy = (float)(t / l0), cz = (float)(i / (l0 * l1));
    const uint32_t nm = *count;
    const size_t N = L.n;
    float acc = 0.0f;
    for (uint32_t base = 0; base < nm; base += MAG_TILE) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < MAG_TILE && base + k < nm; k += blockDim.x) {
            const uint32_t m = mags[base + k];
            uint32_t x, y, z;
            cell_xyz(L, m, x, y, z);
            s_p[k] = make_float4((float)(x + 1u), (float)(y + 1u), (float)(z + 1u), 0.0f);
            s_m[k] = make_float4(L.b_dyn[m], L.b_dyn[N + m], L.b_dyn[2 * N + m], 0.0f);
        }
        __syncthreads();
        const uint32_t cnt = min(MAG_TILE, nm - base);
        if (i < np) {
            for (uint32_t k = 0; k < cnt; k++) {
                const float4 p = s_p[k], m = s_m[k];
                const float dx = cx - p.x, dy = cy - p.y, dz = cz - p.z;
                const float l = sqrtf((dx * dx + dy * dy) + dz * dz);
                if (!(l == 0.0f)) acc = acc + ((dx * m.x + dy * m.y) + dz * m.z) / ((l * l) * l);
            }
        }
    }
    if (i < np) psi[i] = (float)((double)acc / (4.0 * 3.14159265358979323846));
}

__global__ void __launch_bounds__(256) k_static_b(const DevLbm L, const float* psi) {
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= L.n || (L.flags[n] & F_S) == F_S) return;
    uint32_t x, y, z;
    cell_xyz(L, n, x, y, z);
    const uint32_t l0 = L.nx + 2, l1 = L.ny + 2;
    const size_t c = (x + 1u) + ((size_t)(y + 1u) + (size_t)(z + 1u) * l1) * l0;
    const size_t zo = (size_t)l0 * l1;
    const float gx = (psi[c + 1] - psi[c - 1]) / 2.0f, gy = (psi[c + l0] - psi[c - l0]) / 2.0f,
                gz = (psi[c + zo] - psi[c - zo]) / 2.0f;
    const float m = -L.kmu0;
    const size_t N = L.n;
    L.b_stat[n] = L.b_stat[n] + m * gx;
    L.b_stat[N + n] = L.b_stat[N + n] + m * gy;
    L.b_stat[2 * N + n] = L.b_stat[2 * N + n] + m * gz;
}

void launch_psi_static_b(const DevLbm& L, const uint32_t* mags, const uint32_t* count, cudaStream_t s) {
    const uint64_t np = (uint64_t)(L.nx + 2) * (L.ny + 2) * (L.nz + 2);
    k_psi<<<grid_for(np, 256), 256, 0, s>>>(L, mags, count, L.e_dyn);
    k_static_b<<<grid_for(L.n, 256), 256, 0, s>>>(L, L.e_dyn);
}

// static E from charged solids (charge per cell held in B_dyn.x by the voxeliser) into E:
// E_stat (static_e_from_mesh) or E_var (precompute_E_ECR, the same kernel)
__global__ void __launch_bounds__(256) k_static_e(const DevLbm L, const uint32_t* list, const uint32_t* count, float* E) {
    __shared__ float4 s_c[MAG_TILE];
    const uint32_t n = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = n < L.n && (L.flags[n] & F_S) != F_S;
    uint32_t x = 0, y = 0, z = 0;
    if (n < L.n) cell_xyz(L, n, x, y, z);
    const uint32_t nc = *count;
    float ex = 0.0f, ey = 0.0f, ez = 0.0f;
    for (uint32_t base = 0; base < nc; base += MAG_TILE) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < MAG_TILE && base + k < nc; k += blockDim.x) {
            const uint32_t m = list[base + k];
            uint32_t a, b, c;
            cell_xyz(L, m, a, b, c);
            s_c[k] = make_float4((float)a, (float)b, (float)c, L.b_dyn[m]);
        }
        __syncthreads();
        if (active) {
            const uint32_t cnt = min(MAG_TILE, nc - base);
            for (uint32_t k = 0; k < cnt; k++) {
                const float4 p = s_c[k];
                const float dx = (float)x - p.x, dy = (float)y - p.y, dz = (float)z - p.z;
                const float l = sqrtf((dx * dx + dy * dy) + dz * dz);
                if (l == 0.0f) continue;
                const float l3 = (l * l) * l;
                ex = ex + (dx * p.w) / l3; ey = ey + (dy * p.w) / l3; ez = ez + (dz * p.w) / l3;
            }
        }
    }
    if (active) {
        const size_t N = L.n;
        E[n] = E[n] + ex * L.ke;
        E[N + n] = E[N + n] + ey * L.ke;
        E[2 * N + n] = E[2 * N + n] + ez * L.ke;
    }
}

void launch_static_e(const DevLbm& L, const uint32_t* list, const uint32_t* count, float* E, cudaStream_t s) {
    k_static_e<<<grid_for(L.n, 256), 256, 0, s>>>(L, list, count, E);
}

void launch_sum_f64(const void* x, int ft, uint64_t count, double* partials, uint32_t nparts, double* out,
                    cudaStream_t s) {
    // nparts blocks of ceil(count / nparts) values (reduce_f64.cuh)
    launch_sum_two_pass(x, ft, count, (count + nparts - 1) / nparts, nparts, partials, out, s);
}

// ---------------------------------------------------------------------------
// storage-codec round trip (used to check the device codecs exhaustively)
// ---------------------------------------------------------------------------
__global__ void k_codec(int ft, const float* in, uint16_t* enc, float* dec, const uint16_t* raw, float* raw_dec,
                        uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (ft == ION_FP16S) {
        Ddf<ION_FP16S>::st(enc, i, in[i]);
        dec[i] = Ddf<ION_FP16S>::ld(enc, i);
        raw_dec[i] = Ddf<ION_FP16S>::ld(raw, i);
    } else {
        Ddf<ION_FP16C>::st(enc, i, in[i]);
        dec[i] = Ddf<ION_FP16C>::ld(enc, i);
        raw_dec[i] = Ddf<ION_FP16C>::ld(raw, i);
    }
}

void launch_codec(int ft, const float* in, uint16_t* enc, float* dec, const uint16_t* raw, float* raw_dec, uint64_t n,
                  cudaStream_t s) {
    k_codec<<<grid_for(n, 256), 256, 0, s>>>(ft, in, enc, dec, raw, raw_dec, n);
}

// ---------------------------------------------------------------------------
// FP32 FMA throughput probe: 8 independent FMA chains per thread, enough
// warps to fill every SM; the denominator of the field kernel's roofline.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_fma_probe(float* out, int iters, float a, float b) {
    float r[8];
#pragma unroll
    for (int k = 0; k < 8; k++) r[k] = (float)(threadIdx.x + k) * 1e-3f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) r[k] = fmaf(r[k], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; k++) s += r[k];
    if (s == 123.456f) out[threadIdx.x] = s;  // keeps the chains alive
}

// ---------------------------------------------------------------------------
// Self-test of div_rn_shared against the IEEE division, bit for bit, on
// pseudo-random quotients over the ranges the E/B sums produce: numerators
// |x| in [2^-1, 2^13) and exact small integers and halves, denominators
// b = (s s) s with s = sqrt(r2), r2 in [2^-2, 2^27), and b drawn directly in
// [2^-3, 2^40).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ float unit(uint64_t v) { return (float)(v >> 40) * (1.0f / 16777216.0f); }  // [0, 1)

__global__ void __launch_bounds__(256) k_div_check(uint64_t samples, uint64_t seed, unsigned long long* bad,
                                                   float* first_bad) {
    unsigned long long local = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < samples;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h1 = mix64(seed ^ (i * 3 + 0)), h2 = mix64(seed ^ (i * 3 + 1)), h3 = mix64(seed ^ (i * 3 + 2));
        float x;
        if ((h1 & 7u) == 0) x = (float)((int)(h1 >> 40) % 16385 - 8192) * 0.5f;  // small integers and halves
        else x = exp2f(-1.0f + 14.0f * unit(h1)) * ((h1 & 8u) ? -1.0f : 1.0f);
        float b;
        if (h2 & 1u) {
            const float s = sqrtf(exp2f(-2.0f + 29.0f * unit(h2)));
            b = (s * s) * s;
        } else {
            b = exp2f(-3.0f + 43.0f * unit(h2));
        }
        b = __uint_as_float(__float_as_uint(b) ^ ((uint32_t)h3 & 0x7u));  // vary the low mantissa bits
        const float want = __fdiv_rn(x, b);
        const float got = div_rn_shared(x, b, __frcp_rn(b));
        if (__float_as_uint(want) != __float_as_uint(got)) {
            if (atomicAdd(bad, 1ull) == 0ull) { first_bad[0] = x; first_bad[1] = b; }
            local++;
        }
    }
    (void)local;
}

void launch_div_check(uint64_t samples, uint64_t seed, unsigned long long* bad, float* first_bad, cudaStream_t s) {
    k_div_check<<<152 * 8, 256, 0, s>>>(samples, seed, bad, first_bad);
}

void launch_fma_probe(float* out, int blocks, int iters, cudaStream_t s) {
    k_fma_probe<<<blocks, 256, 0, s>>>(out, iters, 0.999999f, 1e-6f);
}

}  // namespace ion
