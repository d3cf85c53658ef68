// lbm_kernels.cuh -- initialize / stream_collide / update_fields of the
// IonSolver timestep as sm_103a kernels (one thread per cell: grid-stride over
// the cells, or over x-rows staged in shared memory for D3Q19 stream_collide).
//
// Per cell the arithmetic follows the reference kernel operation for
// operation (IonSolver src/kernels/sim_kernels.cl:465-859), so results are
// bit-identical to it when it runs in cell order; with -fmad=false no
// product is fused unless the reference calls fma().  The one structural
// change is the LOD accumulation (sim_kernels.cl:666-677): instead of four
// float atomics per cell, each cell stores its velocity contribution and a
// separate pass (field_kernels.cu) sums every bin in ascending cell order.
#pragma once
#include <algorithm>
#include <mutex>

#include "ion_device.cuh"
#include "ion_launch.h"

namespace ion {

// Esoteric-Pull neighbour index for direction i (periodic, sim_kernels.cl:248-302)
struct Nbr {
    uint32_t x0, xp, xm, y0, yp, ym, z0, zp, zm;  // x, and y*nx / z*nx*ny offsets
    __device__ __forceinline__ Nbr(const DevLbm& L, uint32_t x, uint32_t y, uint32_t z) {
        const uint32_t nxy = L.nx * L.ny;
        x0 = x; xp = (x + 1u == L.nx) ? 0u : x + 1u; xm = (x == 0u) ? L.nx - 1u : x - 1u;
        y0 = y * L.nx; yp = ((y + 1u == L.ny) ? 0u : y + 1u) * L.nx; ym = ((y == 0u) ? L.ny - 1u : y - 1u) * L.nx;
        z0 = z * nxy; zp = ((z + 1u == L.nz) ? 0u : z + 1u) * nxy; zm = ((z == 0u) ? L.nz - 1u : z - 1u) * nxy;
    }
    template <class V>
    __device__ __forceinline__ uint32_t operator()(int i) const {
        const int cx = V::c(i, 0), cy = V::c(i, 1), cz = V::c(i, 2);
        return (cx > 0 ? xp : cx < 0 ? xm : x0) + (cy > 0 ? yp : cy < 0 ? ym : y0) + (cz > 0 ? zp : cz < 0 ? zm : z0);
    }
};

// density / velocity from DDF-shifted populations (sim_kernels.cl:208-233)
template <class V>
__device__ __forceinline__ void moments(const float* f, float& rho, float& ux, float& uy, float& uz) {
    float r = f[0];
#pragma unroll
    for (int i = 1; i < V::q; i++) r = r + f[i];
    r = r + 1.0f;
    float u[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        bool first = true;
        float acc = 0.0f;
#pragma unroll
        for (int i = 1; i < V::q; i += 2) {
            const int s = V::c(i, a);
            if (s == 0) continue;
            const float pos = s > 0 ? f[i] : f[i + 1], neg = s > 0 ? f[i + 1] : f[i];
            acc = first ? pos - neg : (acc + pos) - neg;
            first = false;
        }
        u[a] = acc;
    }
    rho = r;
    ux = u[0] / r;
    uy = u[1] / r;
    uz = (V::dims == 2 ? 0.0f : u[2]) / r;
}

// c_i . v over the non-zero components in x,y,z order (sim_kernels.cl:162-205)
template <class V>
__device__ __forceinline__ float project(int i, float vx, float vy, float vz) {
    bool first = true;
    float acc = 0.0f;
    const float comp[3] = {vx, vy, vz};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int s = V::c(i, a);
        if (s == 0) continue;
        if (first) { acc = s > 0 ? comp[a] : -comp[a]; first = false; }
        else acc = s > 0 ? acc + comp[a] : acc - comp[a];
    }
    return acc;
}

// equilibrium, DDF-shifted (sim_kernels.cl:155-207)
template <class V>
__device__ __forceinline__ void equilibrium(float rho, float ux, float uy, float uz, float* feq) {
    const float c3 = -3.0f * ((ux * ux + uy * uy) + uz * uz), rm1 = rho - 1.0f;
    ux = ux * 3.0f; uy = uy * 3.0f; uz = uz * 3.0f;
    feq[0] = V::w(0) * fmaf(rho, 0.5f * c3, rm1);
#pragma unroll
    for (int i = 1; i < V::q; i += 2) {
        const float wr = V::w(V::wc(i)) * rho, wrm1 = V::w(V::wc(i)) * rm1;
        const float p = project<V>(i, ux, uy, uz);
        feq[i] = fmaf(wr, fmaf(0.5f, fmaf(p, p, c3), p), wrm1);
        feq[i + 1] = fmaf(wr, fmaf(0.5f, fmaf(p, p, c3), -p), wrm1);
    }
}

// Guo forcing terms (sim_kernels.cl:367-377)
template <class V>
__device__ __forceinline__ void forcing(float ux, float uy, float uz, float fx, float fy, float fz, float* Fin) {
    const float uF = V::dims == 2 ? -THIRD * fmaf(ux, fx, uy * fy) : -THIRD * fmaf(ux, fx, fmaf(uy, fy, uz * fz));
    Fin[0] = (9.0f * V::w(0)) * uF;
#pragma unroll
    for (int i = 1; i < V::q; i++) {
        const float cx = (float)V::c(i, 0), cy = (float)V::c(i, 1), cz = (float)V::c(i, 2);
        const float cf = (cx * fx + cy * fy) + cz * fz;
        const float cu = ((cx * ux + cy * uy) + cz * uz) + THIRD;
        Fin[i] = (9.0f * V::w(V::wc(i))) * fmaf(cf, cu, uF);
    }
}

// D3Q7 advection equilibrium (sim_kernels.cl:390-396)
__device__ __forceinline__ void adv_equilibrium(float Q, float ux, float uy, float uz, float* a) {
    const float hq = 0.5f * Q, eq = 0.125f * (Q - 1.0f);
    a[0] = fmaf(0.25f, Q, -0.25f);
    a[1] = fmaf(hq, ux, eq); a[2] = fmaf(hq, -ux, eq);
    a[3] = fmaf(hq, uy, eq); a[4] = fmaf(hq, -uy, eq);
    a[5] = fmaf(hq, uz, eq); a[6] = fmaf(hq, -uz, eq);
}

// Esoteric-Pull load/store (sim_kernels.cl:234-247, 397-410)
template <class D, int Q, class NB>
__device__ __forceinline__ void ep_load(const typename D::T* f, uint32_t N, uint32_t n, bool odd, const NB& j, float* v) {
    v[0] = D::ld(f, n);
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
        v[i] = D::ld(f, (size_t)(odd ? i : i + 1) * N + n);
        v[i + 1] = D::ld(f, (size_t)(odd ? i + 1 : i) * N + j(i));
    }
}
// Where a cell's new DDFs go (Esoteric-Pull, sim_kernels.cl:397-410): DDF 0 to slot
// 0 of the cell (st0), the DDF of odd direction i to slot odd ? i + 1 : i of the
// neighbour in direction i (st_nbr), that of direction i + 1 to slot odd ? i : i + 1
// of the cell (st_own) -- exactly the locations the cell read its DDFs from.
// GlobalDst computes the addresses; IX is the type the slot offsets are computed in
// (uint32_t where Q N < 2^32 is known).
template <class D, class NB, class IX = size_t>
struct GlobalDst {
    typename D::T* f;
    uint32_t N, n;
    bool odd;
    const NB& j;
    __device__ __forceinline__ void st0(float v) const { D::st(f, n, v); }
    __device__ __forceinline__ void st_nbr(int i, float v) const { D::st(f, (IX)(odd ? i + 1 : i) * N + j(i), v); }
    __device__ __forceinline__ void st_own(int i, float v) const { D::st(f, (IX)(odd ? i : i + 1) * N + n, v); }
};
template <int Q, class DST>
__device__ __forceinline__ void ep_store_to(const DST& o, const float* v) {
    o.st0(v[0]);
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
        o.st_nbr(i, v[i]);
        o.st_own(i, v[i + 1]);
    }
}
template <class D, int Q, class NB, class IX = size_t>
__device__ __forceinline__ void ep_store(typename D::T* f, uint32_t N, uint32_t n, bool odd, const NB& j, const float* v) {
    ep_store_to<Q>(GlobalDst<D, NB, IX>{f, N, n, odd, j}, v);
}

// L2 prefetch of the slots ep_load will read (no registers held; the later
// loads then wait on L2 instead of DRAM)
template <class T, int Q, class NB>
__device__ __forceinline__ void ep_prefetch(const T* f, uint32_t N, uint32_t n, bool odd, const NB& j) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(f + n));
#pragma unroll
    for (int i = 1; i < Q; i += 2) {
        asm volatile("prefetch.global.L2 [%0];" ::"l"(f + (size_t)(odd ? i : i + 1) * N + n));
        asm volatile("prefetch.global.L2 [%0];" ::"l"(f + (size_t)(odd ? i + 1 : i) * N + j(i)));
    }
}

template <class V>
struct NbV {  // neighbour functor of a velocity set
    const Nbr& b;
    __device__ __forceinline__ uint32_t operator()(int i) const { return b.template operator()<V>(i); }
};
struct Nb7 {  // D3Q7 subset (sim_kernels.cl:382-389)
    const Nbr& b;
    __device__ __forceinline__ uint32_t operator()(int i) const {
        return i == 1 ? b.xp + b.y0 + b.z0 : i == 3 ? b.x0 + b.yp + b.z0 : b.x0 + b.y0 + b.zp;
    }
};

// Where sc_cell reads a cell's inputs.  Both sources return the same values, so
// the arithmetic (and its results) do not depend on the choice.
enum { LAT_FI = 0, LAT_EI = 1, LAT_FQI = 2 };
// straight from global memory (Esoteric-Pull addressing, sim_kernels.cl:234-247)
struct GlobalSrc {
    static constexpr bool prefetch = true;
    __device__ __forceinline__ uint8_t flags(const DevLbm& L, uint32_t n) const { return L.flags[n]; }
    // c = 0..2: B_dyn x, y, z; 3..5: E_dyn x, y, z
    __device__ __forceinline__ float eb(const DevLbm& L, int c, uint32_t n) const {
        return c < 3 ? L.b_dyn[(size_t)c * L.n + n] : L.e_dyn[(size_t)(c - 3) * L.n + n];
    }
    template <class D, int Q, class NB>
    __device__ __forceinline__ void load(const typename D::T* f, uint32_t N, uint32_t n, bool odd, const NB& j,
                                         float* v, int) const {
        ep_load<D, Q>(f, N, n, odd, j, v);
    }
    template <class D, int Q, class IX, class NB>
    __device__ __forceinline__ GlobalDst<D, NB, IX> dst(typename D::T* f, uint32_t N, uint32_t n, bool odd, const NB& j,
                                                        int) const {
        return {f, N, n, odd, j};
    }
};
// D3Q19 offsets (in rows) of the staged streams of each lattice: fi 19, ei 19, fqi 7
__host__ __device__ constexpr uint32_t row_stream_base(int lat) { return lat == LAT_FI ? 0u : lat == LAT_EI ? 19u : 38u; }
// x shift of the neighbour row read for direction i (i odd) of a D3Q19 or D3Q7 lattice
template <int Q>
__host__ __device__ constexpr int row_cx(int i) { return Q == 7 ? (i == 1 ? 1 : 0) : VSet<19>::c(i, 0); }

// A cell's new DDFs into the staged row they were read from (the cell's stores land
// exactly on its loads, see GlobalDst): stream i at x for st_own, stream i + 1 at the
// x of the neighbour for st_nbr.  RS: the row stride in elements (0: nx).
template <class D, int Q, uint32_t RS>
struct RowDst {
    typename D::T* r;  // the lattice's stream 0
    uint32_t nx, x, xp, xm;
    __device__ __forceinline__ uint32_t stride() const { return RS ? RS : nx; }
    __device__ __forceinline__ void st0(float v) const { r[x] = D::enc(v); }
    __device__ __forceinline__ void st_own(int i, float v) const { r[(uint32_t)i * stride() + x] = D::enc(v); }
    __device__ __forceinline__ void st_nbr(int i, float v) const {
        const int cx = row_cx<Q>(i);
        r[(uint32_t)(i + 1) * stride() + (cx > 0 ? xp : cx < 0 ? xm : x)] = D::enc(v);
    }
};

// From one x-row staged in shared memory by the row kernels: stream s of a lattice
// holds the row that DDF s of every cell of the row is read from (stream 0 and the
// odd streams: the cell's own row; stream i + 1: the row of the neighbour in direction
// i, read at the neighbour's x), then the E/B rows and the flags row.  RS: the row
// stride in elements (0: nx).  WB: the new DDFs are written back into the staged rows
// (the kernel then copies the rows back to global memory) instead of to global memory.
template <class T, uint32_t RS = 0, bool WB = false>
struct RowSrc {
    static constexpr bool prefetch = false;
    uint8_t* buf;
    uint32_t nx, x, xp, xm, eb_off, fl_off;
    __device__ __forceinline__ uint32_t stride() const { return RS ? RS : nx; }
    __device__ __forceinline__ uint8_t flags(const DevLbm&, uint32_t) const { return buf[fl_off + x]; }
    __device__ __forceinline__ float eb(const DevLbm&, int c, uint32_t) const {
        return reinterpret_cast<const float*>(buf + eb_off)[(uint32_t)c * stride() + x];
    }
    template <class D, int Q, class NB>
    __device__ __forceinline__ void load(const T*, uint32_t, uint32_t, bool, const NB&, float* v, int lat) const {
        const T* r = reinterpret_cast<const T*>(buf) + row_stream_base(lat) * stride();
        v[0] = D::dec(r[x]);
#pragma unroll
        for (int i = 1; i < Q; i += 2) {
            const int cx = row_cx<Q>(i);
            v[i] = D::dec(r[(uint32_t)i * stride() + x]);
            v[i + 1] = D::dec(r[(uint32_t)(i + 1) * stride() + (cx > 0 ? xp : cx < 0 ? xm : x)]);
        }
    }
    template <class D, int Q, class IX, class NB>
    __device__ __forceinline__ auto dst(typename D::T* f, uint32_t N, uint32_t n, bool odd, const NB& j, int lat) const {
        if constexpr (WB)
            return RowDst<D, Q, RS>{reinterpret_cast<T*>(buf) + row_stream_base(lat) * stride(), nx, x, xp, xm};
        else
            return GlobalDst<D, NB, IX>{f, N, n, odd, j};
    }
};

// ---------------------------------------------------------------------------
// Fused equilibrium / forcing / collision / store, one direction pair at a
// time.  Each value is computed with exactly the operations of
// equilibrium() / forcing() above and of the reference's collision loops
// (sim_kernels.cl:714-754); only the order in which independent directions
// are finished changes, which keeps far fewer values live in registers.
// ---------------------------------------------------------------------------
struct EqState {
    float rho, rm1, c3, ux, uy, uz;  // u already multiplied by 3
};
__device__ __forceinline__ EqState eq_state(float rho, float ux, float uy, float uz) {
    EqState s;
    s.c3 = -3.0f * ((ux * ux + uy * uy) + uz * uz);
    s.rm1 = rho - 1.0f;
    s.rho = rho;
    s.ux = ux * 3.0f; s.uy = uy * 3.0f; s.uz = uz * 3.0f;
    return s;
}
template <class V>
__device__ __forceinline__ float eq_zero(const EqState& s) { return V::w(0) * fmaf(s.rho, 0.5f * s.c3, s.rm1); }
template <class V>
__device__ __forceinline__ void eq_pair(const EqState& s, int i, float& a, float& b) {
    const float wr = V::w(V::wc(i)) * s.rho, wrm1 = V::w(V::wc(i)) * s.rm1;
    const float p = project<V>(i, s.ux, s.uy, s.uz);
    a = fmaf(wr, fmaf(0.5f, fmaf(p, p, s.c3), p), wrm1);
    b = fmaf(wr, fmaf(0.5f, fmaf(p, p, s.c3), -p), wrm1);
}
struct ForceState {
    float ux, uy, uz, fx, fy, fz, uF;
};
template <class V>
__device__ __forceinline__ ForceState force_state(float ux, float uy, float uz, float fx, float fy, float fz) {
    ForceState s{ux, uy, uz, fx, fy, fz, 0.0f};
    s.uF = V::dims == 2 ? -THIRD * fmaf(ux, fx, uy * fy) : -THIRD * fmaf(ux, fx, fmaf(uy, fy, uz * fz));
    return s;
}
template <class V>
__device__ __forceinline__ float force_dir(const ForceState& s, int i) {
    if (i == 0) return (9.0f * V::w(0)) * s.uF;
    const float cx = (float)V::c(i, 0), cy = (float)V::c(i, 1), cz = (float)V::c(i, 2);
    const float cf = (cx * s.fx + cy * s.fy) + cz * s.fz;
    const float cu = ((cx * s.ux + cy * s.uy) + cz * s.uz) + THIRD;
    return (9.0f * V::w(V::wc(i))) * fmaf(cf, cu, s.uF);
}

// SRT collision + Esoteric-Pull store (sim_kernels.cl:714-723 / 649-656).
// force: 0 = none (Fin = 0), 1 = Guo terms scaled by c_tau.
template <class V, class DST>
__device__ __forceinline__ void srt_store(const DST& o, const float* fh, const EqState& es, const ForceState& fs,
                                          bool force, float c_tau, float w, bool eqc) {
    {
        const float feq = eq_zero<V>(es);
        const float F = force ? force_dir<V>(fs, 0) * c_tau : 0.0f;
        o.st0(eqc ? feq : fmaf(1.0f - w, fh[0], fmaf(w, feq, F)));
    }
#pragma unroll
    for (int i = 1; i < V::q; i += 2) {
        float fa, fb;
        eq_pair<V>(es, i, fa, fb);
        const float Fa = force ? force_dir<V>(fs, i) * c_tau : 0.0f;
        const float Fb = force ? force_dir<V>(fs, i + 1) * c_tau : 0.0f;
        const float va = eqc ? fa : fmaf(1.0f - w, fh[i], fmaf(w, fa, Fa));
        const float vb = eqc ? fb : fmaf(1.0f - w, fh[i + 1], fmaf(w, fb, Fb));
        o.st_nbr(i, va);
        o.st_own(i, vb);
    }
}

// TRT collision + store (sim_kernels.cl:725-754)
template <class V, class DST>
__device__ __forceinline__ void trt_store(const DST& o, const float* fh, const EqState& es, const ForceState& fs,
                                          bool force, float w, bool eqc) {
    const float wp = w, wm = 1.0f / (0.1875f / (1.0f / w - 0.5f) + 0.5f);
    const float ctp = fmaf(wp, -0.25f, 0.5f), ctm = fmaf(wm, -0.25f, 0.5f);
    {
        const float feq = eq_zero<V>(es);
        float F = 0.0f;
        if (force) {
            const float F0 = force_dir<V>(fs, 0);
            F = fmaf(ctp, F0 + F0, ctm * (F0 - F0));
        }
        const float sym = ((feq - fh[0]) + feq) - fh[0];
        const float asym = ((feq - feq) - fh[0]) + fh[0];
        o.st0(eqc ? feq : fmaf(0.5f * wp, sym, fmaf(0.5f * wm, asym, fh[0] + F)));
    }
#pragma unroll
    for (int i = 1; i < V::q; i += 2) {
        float ea, eb;
        eq_pair<V>(es, i, ea, eb);
        float Fa = 0.0f, Fb = 0.0f;
        if (force) {
            const float A = force_dir<V>(fs, i), B = force_dir<V>(fs, i + 1);
            Fa = fmaf(ctp, A + B, ctm * (A - B));
            Fb = fmaf(ctp, B + A, ctm * (B - A));
        }
        const float ha = fh[i], hb = fh[i + 1];
        const float va = eqc ? ea : fmaf(0.5f * wp, ((ea - ha) + eb) - hb, fmaf(0.5f * wm, ((ea - eb) - ha) + hb, ha + Fa));
        const float vb = eqc ? eb : fmaf(0.5f * wp, ((eb - hb) + ea) - ha, fmaf(0.5f * wm, ((eb - ea) - hb) + ha, hb + Fb));
        o.st_nbr(i, va);
        o.st_own(i, vb);
    }
}

// ---------------------------------------------------------------------------
// stream_collide, one step (sim_kernels.cl:465-758)
// ---------------------------------------------------------------------------
// SUBGRID_ECR (sim_kernels.cl:449-462): |V| at cell m and the gradient of |B_dyn|
// with the reference's expression a - b / 2 per axis; zero on the domain border
__device__ __forceinline__ float mag_v(const float* V, size_t N, uint32_t m) {
    return sqrtf((V[m] * V[m] + V[N + m] * V[N + m]) + V[2 * N + m] * V[2 * N + m]);
}

template <int Q, int FT, bool MHD, bool TRT, bool ECR = false, class SRC = GlobalSrc, class IX = size_t>
__device__ __forceinline__ void sc_cell(const DevLbm& L, const uint32_t n, const bool odd, const SRC& S = SRC{}) {
    using V = VSet<Q>;
    using D = Ddf<FT>;
    using T = typename D::T;
    const uint32_t N = L.n;
    const uint8_t fbo = S.flags(L, n) & F_BO;
    if (fbo == F_S) return;
    const bool eqc = L.ext_eq && fbo == F_E;
    uint32_t x, y, z;
    cell_xyz(L, n, x, y, z);
    const Nbr nb(L, x, y, z);
    const NbV<V> j{nb};
    const float w = L.w;
    const float c_tau = fmaf(w, -0.5f, 1.0f);
    float rhoe = 0.0f, Bx = 0.0f, By = 0.0f, Bz = 0.0f, Ex = 0.0f, Ey = 0.0f, Ez = 0.0f, dq_ecr = 0.0f;
    if constexpr (MHD) {
        // the gas and charge lattices are read after the electron gas: start them towards L2
        if constexpr (SRC::prefetch) {
            ep_prefetch<T, Q>((const T*)L.fi, N, n, odd, j);
            ep_prefetch<T, 7>((const T*)L.fqi, N, n, odd, Nb7{nb});
        }
        Bx = S.eb(L, 0, n); By = S.eb(L, 1, n); Bz = S.eb(L, 2, n);
        Ex = S.eb(L, 3, n); Ey = S.eb(L, 4, n); Ez = S.eb(L, 5, n);
    }
    // MHD: the electron gas first (pass 0), then the gas (pass 1).  The electron gas
    // reads no value of the gas lattice, so its DDFs are dead before the gas DDFs load
    // (fewer registers live at once).  With FP16C storage both passes run one copy of the
    // load, moments, collision and store code (the loop is not unrolled): the integer
    // codec makes the unrolled cell too large for the instruction cache, and sharing
    // measured 11% faster at 256^3; FP32 and FP16S keep the unrolled form (the shared
    // one measured equal and 2.5% slower).  Each pass computes exactly the values of
    // the reference's code for its lattice.
#pragma unroll(FT == ION_FP16C ? 1 : 2)
    for (int pass = MHD ? 0 : 1; pass < 2; pass++) {
        const bool electrons = MHD && pass == 0;
        T* const f = (T*)(electrons ? L.ei : L.fi);
        const int lat = electrons ? LAT_EI : LAT_FI;
        float fh[Q];
        S.template load<D, Q>(f, N, n, odd, j, fh, lat);
        float rho, ux, uy, uz, fx, fy, fz;
        bool force;
        if (!electrons && eqc) { rho = L.rho[n]; ux = L.u[n]; uy = L.u[(size_t)N + n]; uz = L.u[2 * (size_t)N + n]; }
        else moments<V>(fh, rho, ux, uy, uz);
        if (electrons) {
            // electron gas: Lorentz force, Guo half-step (sim_kernels.cl:530-656)
            if constexpr (ECR) {  // SUBGRID_ECR, sim_kernels.cl:564-628 (the ionisation term is the reference's placeholder)
                const Nb7 j7{nb};
                float ethn[7];
                ep_load<D, 7>((const T*)L.eti, N, n, odd, j7, ethn);
                float Etn = 0.0f;
#pragma unroll
                for (int i = 0; i < 7; i++) Etn = Etn + ethn[i];
                Etn = Etn + 1.0f;
                // ECR heating by the oscillating field's part perpendicular to B
                const float Evx = L.e_var[n], Evy = L.e_var[(size_t)N + n], Evz = L.e_var[2 * (size_t)N + n];
                const float lB = sqrtf((Bx * Bx + By * By) + Bz * Bz);
                const float kpar = ((Evx * Bx + Evy * By) + Evz * Bz) / (lB * lB);
                const float pex = Evx - kpar * Bx, pey = Evy - kpar * By, pez = Evz - kpar * Bz;
                const float Emag = sqrtf((pex * pex + pey * pey) + pez * pez);
                Etn = Etn + (((L.keabs / L.kkbme) * (rho + 0.00001f)) / L.kkge) * (Emag * Emag);
                // guiding-centre drift along -grad |B|
                float gx = 0.0f, gy = 0.0f, gz = 0.0f;
                if (!(x == 0u || x == L.nx - 1u || y == 0u || y == L.ny - 1u || z == 0u || z == L.nz - 1u)) {
                    const uint32_t sx = 1u, sy = L.nx, sz = L.nx * L.ny;
                    gx = mag_v(L.b_dyn, N, n + sx) - mag_v(L.b_dyn, N, n - sx) / 2.0f;
                    gy = mag_v(L.b_dyn, N, n + sy) - mag_v(L.b_dyn, N, n - sy) / 2.0f;
                    gz = mag_v(L.b_dyn, N, n + sz) - mag_v(L.b_dyn, N, n - sz) / 2.0f;
                }
                const float kt = L.kkbme * Etn;
                const float dux = (kt * gx) / lB, duy = (kt * gy) / lB, duz = (kt * gz) / lB;
                ux = ux + dux;
                uy = uy + duy;
                uz = uz + duz;
                Etn = Etn - sqrtf((dux * dux + duy * duy) + duz * duz) / L.kkbme;
                float eteq[7];
                adv_equilibrium(Etn, ux, uy, uz, eteq);
                if (L.update_fields) L.et[n] = Etn;
#pragma unroll
                for (int i = 0; i < 7; i++) ethn[i] = fmaf(1.0f - L.wq, ethn[i], L.wq * eteq[i]);
                ep_store<D, 7>((T*)L.eti, N, n, odd, j7, ethn);
                dq_ecr = 0.0001f * Etn;  // ionisation: added to the electron and the gas charge
                rho = rho + dq_ecr;
            }
            const float cxv = uy * Bz - uz * By, cyv = uz * Bx - ux * Bz, czv = ux * By - uy * Bx;
            const float nre = -rho;
            fx = nre * (Ex + cxv); fy = nre * (Ey + cyv); fz = nre * (Ez + czv);
            const float r2e = 0.5f / (rho * L.kkge);
            ux = clampf(fmaf(fx, r2e, ux), -CS, CS);
            uy = clampf(fmaf(fy, r2e, uy), -CS, CS);
            uz = clampf(fmaf(fz, r2e, uz), -CS, CS);
            rhoe = rho;
            force = true;
        } else {
            fx = L.fx; fy = L.fy; fz = L.fz;
            if (L.ext_ff) { fx = fx + L.F[n]; fy = fy + L.F[(size_t)N + n]; fz = fz + L.F[2 * (size_t)N + n]; }
            if constexpr (MHD) {
                // charge advection (D3Q7): load, charge, collide, store
                const Nb7 j7{nb};
                float rhoq;
                {
                    float qhn[7];
                    S.template load<D, 7>((const T*)L.fqi, N, n, odd, j7, qhn, LAT_FQI);
                    rhoq = 0.0f;
#pragma unroll
                    for (int i = 0; i < 7; i++) rhoq = rhoq + qhn[i];
                    rhoq = rhoq + 1.0f;
                    if constexpr (ECR) rhoq = rhoq + dq_ecr;
                    float aeq[7];
                    adv_equilibrium(rhoq, ux, uy, uz, aeq);
#pragma unroll
                    for (int i = 0; i < 7; i++) qhn[i] = fmaf(1.0f - L.wq, qhn[i], L.wq * aeq[i]);
                    ep_store_to<7>(S.template dst<D, 7, IX>((T*)L.fqi, N, n, odd, j7, LAT_FQI), qhn);
                }
                L.q[n] = rhoq - rhoe;
                // Lorentz force on the gas
                fx = fx + rhoq * ((Ex + uy * Bz) - uz * By);
                fy = fy + rhoq * ((Ey + uz * Bx) - ux * Bz);
                fz = fz + rhoq * ((Ez + ux * By) - uy * Bx);
                // LOD contribution: velocity / bin volume (the charge is q[n])
                if (L.depth > 0u) {
                    L.lod_cell[n] = ux * L.ils;
                    L.lod_cell[(size_t)N + n] = uy * L.ils;
                    L.lod_cell[2 * (size_t)N + n] = uz * L.ils;
                }
            }
            if (L.ext_vf) {
                const float r2 = 0.5f / rho;
                ux = clampf(fmaf(fx, r2, ux), -CS, CS);
                uy = clampf(fmaf(fy, r2, uy), -CS, CS);
                uz = clampf(fmaf(fz, r2, uz), -CS, CS);
            } else {
                ux = clampf(ux, -CS, CS);
                uy = clampf(uy, -CS, CS);
                uz = clampf(uz, -CS, CS);
            }
            if (L.update_fields && !eqc) {
                L.rho[n] = rho;
                L.u[n] = ux; L.u[(size_t)N + n] = uy; L.u[2 * (size_t)N + n] = uz;
            }
            force = L.ext_vf;
        }
        const EqState es = eq_state(rho, ux, uy, uz);
        const ForceState fs = force_state<V>(ux, uy, uz, fx, fy, fz);
        const auto dst = S.template dst<D, Q, IX>(f, N, n, odd, j, lat);
        if (TRT && !electrons) trt_store<V>(dst, fh, es, fs, force, w, eqc);
        else srt_store<V>(dst, fh, es, fs, force, c_tau, w, eqc);
    }
}

template <int Q, int FT, bool MHD, bool TRT, bool ECR = false>
__global__ void __launch_bounds__(256, MHD ? 2 : 4) k_stream_collide(const DevLbm L, const uint32_t odd_t) {
    const bool odd = odd_t != 0u;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < L.n; n += gridDim.x * blockDim.x)
        sc_cell<Q, FT, MHD, TRT, ECR>(L, n, odd);
}

// ---------------------------------------------------------------------------
// D3Q19 stream_collide over x-rows staged in shared memory.  Each CTA walks rows
// (y, z) = blockIdx.x, blockIdx.x + gridDim.x, ...; for the next row it issues bulk
// asynchronous copies (cp.async.bulk, completion on the buffer's mbarrier) of every
// stream the row's cells read -- per lattice the own-row slot of DDF 0 and of each
// odd direction, and for each even direction the slot row of the neighbour in the
// pair's direction (periodic in y and z; the x shift is applied when reading) --
// plus the E/B and flag rows, while the row before is computed from the other
// buffer.  All streams are contiguous rows, so the copies keep tens of KB per SM in
// flight without holding registers.  In Esoteric-Pull every slot is read and
// written by the same cell within a step, so staging a row ahead of its cells'
// stores is safe, and the cells' new DDFs can go back into the staged rows (RowDst):
// once a row is computed, its lattice streams are copied back to their global rows
// with cp.async.bulk (shared -> global), whole rows instead of one 2- or 4-byte store
// per DDF.  The arithmetic is sc_cell's (RowSrc/RowDst only change where values are
// read and written).  Two forms: k_sc_rows_ws (rows of up to 256 cells: a producer
// warp and "full"/"empty" mbarriers, no CTA-wide barrier per row) and k_sc_rows
// (longer rows: thread 0 stages and writes back, a CTA barrier releases the buffer).
// A copy that does not land within the wait limit sets *err and the CTA stops after
// waiting (bounded) for its copies in flight; rows not computed are not written back.
// ---------------------------------------------------------------------------
template <int FT, bool MHD>
__host__ __device__ constexpr uint32_t row_streams() { return MHD ? 45u : 19u; }

template <int FT, bool MHD>
__host__ __device__ inline uint32_t row_bytes(uint32_t nx) {
    using T = typename Ddf<FT>::T;
    return row_streams<FT, MHD>() * nx * (uint32_t)sizeof(T) + (MHD ? 6u * nx * 4u : 0u) + ((nx + 15u) & ~15u);
}

// The global rows of the lattice streams of row r = (y, z), in staging-buffer order:
// op(stream, pointer to the row's first element) for each lattice (gas, then electron
// gas and charge), stream 0 and the odd streams from the own row, stream i + 1 from the
// row of the neighbour in direction i (periodic in y and z).
template <int FT, bool MHD, class OP>
__device__ __forceinline__ void for_row_streams(const DevLbm& L, uint32_t r, bool odd, OP&& op) {
    using V = VSet<19>;
    using T = typename Ddf<FT>::T;
    const uint32_t nx = L.nx, ny = L.ny, nz = L.nz, N = L.n;
    const uint32_t y = r % ny, z = r / ny, own = (y + z * ny) * nx;
    auto lattice = [&](T* f, uint32_t base, int Q) {
        op(base, f + own);
        for (int i = 1; i < Q; i += 2) {
            const int cy = Q == 7 ? (i == 3 ? 1 : 0) : V::c(i, 1), cz = Q == 7 ? (i == 5 ? 1 : 0) : V::c(i, 2);
            const uint32_t yy = cy > 0 ? (y + 1u == ny ? 0u : y + 1u) : cy < 0 ? (y == 0u ? ny - 1u : y - 1u) : y;
            const uint32_t zz = cz > 0 ? (z + 1u == nz ? 0u : z + 1u) : cz < 0 ? (z == 0u ? nz - 1u : z - 1u) : z;
            const uint32_t s_own = odd ? (uint32_t)i : (uint32_t)i + 1u, s_nbr = odd ? (uint32_t)i + 1u : (uint32_t)i;
            op(base + i, f + (size_t)s_own * N + own);
            op(base + i + 1, f + (size_t)s_nbr * N + (yy + zz * ny) * nx);
        }
    };
    lattice((T*)L.fi, row_stream_base(LAT_FI), 19);
    if constexpr (MHD) {
        lattice((T*)L.ei, row_stream_base(LAT_EI), 19);
        lattice((T*)L.fqi, row_stream_base(LAT_FQI), 7);
    }
}

__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)), "r"(bytes)
                 : "memory");
}

// Rows longer than 384 cells: CTAs of at most 256 threads, each thread two or more
// cells of the row; thread 0 stages the next row at the start of each row and a CTA
// barrier releases a buffer.  The new DDFs
// are stored to global memory directly: writing them back through the staged rows,
// as k_sc_rows_ws does, measured slower here (FP16S MHD at 384^3 3.60 -> 4.09 ms, FP32
// MHD at 288^3 2.62 -> 3.54 ms, one CTA per SM), because thread 0 then has to wait
// for the copy-back to read a buffer before it can stage the next row into it.
template <int FT, bool MHD, bool TRT>
__global__ void __launch_bounds__(256, 2) k_sc_rows(const DevLbm L, const uint32_t odd_t, uint32_t* err) {
    using T = typename Ddf<FT>::T;
    extern __shared__ __align__(128) uint8_t rows_smem[];
    __shared__ __align__(8) uint64_t bar[2];
    const bool odd = odd_t != 0u;
    const uint32_t nx = L.nx, ny = L.ny, nrows = ny * L.nz, N = L.n;
    const uint32_t rb = nx * (uint32_t)sizeof(T), RB = row_bytes<FT, MHD>(nx);
    const uint32_t eb_off = row_streams<FT, MHD>() * rb, fl_off = eb_off + (MHD ? 6u * nx * 4u : 0u);
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1u);
        mbar_init(&bar[1], 1u);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // copies of row r into buffer b (one thread)
    auto stage = [&](uint32_t r, uint32_t b) {
        uint8_t* dst = rows_smem + b * RB;
        const uint32_t own = r * nx;
        mbar_expect_tx(&bar[b], RB);
        for_row_streams<FT, MHD>(L, r, odd, [&](uint32_t st, T* g) { bulk_g2s(dst + st * rb, g, rb, &bar[b]); });
        if constexpr (MHD) {
            for (uint32_t c = 0; c < 3; c++) {
                bulk_g2s(dst + eb_off + c * nx * 4u, L.b_dyn + (size_t)c * N + own, nx * 4u, &bar[b]);
                bulk_g2s(dst + eb_off + (3u + c) * nx * 4u, L.e_dyn + (size_t)c * N + own, nx * 4u, &bar[b]);
            }
        }
        bulk_g2s(dst + fl_off, L.flags + own, (nx + 15u) & ~15u, &bar[b]);
    };
    uint32_t k = 0;
    bool ok = true;
    if (threadIdx.x == 0 && blockIdx.x < nrows) stage(blockIdx.x, 0u);
    for (uint32_t r = blockIdx.x; r < nrows; r += gridDim.x, k++) {
        const uint32_t b = k & 1u;
        // the other buffer was released at the end of the previous row
        if (threadIdx.x == 0 && r + gridDim.x < nrows) stage(r + gridDim.x, b ^ 1u);
        ok = mbar_wait(&bar[b], (k >> 1) & 1u, L.wait_limit);
        if (!__syncthreads_and(ok)) break;
        uint8_t* buf = rows_smem + b * RB;
        const uint32_t y = r % ny, z = r / ny;
        for (uint32_t x = threadIdx.x; x < nx; x += blockDim.x) {
            const RowSrc<T> S{buf, nx, x, x + 1u == nx ? 0u : x + 1u, x == 0u ? nx - 1u : x - 1u, eb_off, fl_off};
            sc_cell<19, FT, MHD, TRT, false, RowSrc<T>, uint32_t>(L, x + (y + z * ny) * nx, odd, S);
        }
        __syncthreads();  // buffer b is free
    }
    if (!ok && threadIdx.x == 0) {
        // copies still in flight: this row's and possibly the next one's
        const uint32_t b = k & 1u;
        mbar_wait(&bar[b], (k >> 1) & 1u, WAIT_LIMIT);
        if (blockIdx.x + (k + 1u) * gridDim.x < nrows) mbar_wait(&bar[b ^ 1u], ((k + 1u) >> 1) & 1u, WAIT_LIMIT);
        atomicExch(err, 1u);
    }
}

// waits for an mbarrier phase; gives up after `limit` polls (setting *fail) or as soon
// as another warp has set *fail
__device__ __forceinline__ bool mbar_wait_or_fail(uint64_t* bar, uint32_t parity, volatile uint32_t* fail,
                                                  uint32_t limit) {
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(smem_addr(bar)), "r"(parity) : "memory");
        if (done) return true;
        if ((i & 255u) == 255u && *fail) return false;
    }
    *fail = 1u;
    return false;
}

// Rows of up to 384 cells (WS_ROW): blockDim.x = compute threads + 32.  The last warp
// stages rows and writes them back; the others compute (one cell per thread and row).
// The row buffer has a fixed stride of RS elements per stream (the smallest of 128, 256
// and 384 that holds the row: a small buffer keeps more CTAs per SM), so every
// shared-memory access of a cell is a register plus a constant offset.  The cells' new
// DDFs go into the staged rows they were read from (RowDst), and the producer copies
// each finished row's lattice streams back to their global rows with cp.async.bulk
// (shared -> global): a row's streams are read and written by that row's cells only,
// so no other CTA touches them within the step.  The other outputs (q, the LOD
// velocity, rho, u) are stored directly.
constexpr uint32_t WS_ROW = 384;
__host__ __device__ constexpr uint32_t ws_stride(uint32_t nx) { return nx <= 128u ? 128u : nx <= 256u ? 256u : 384u; }
template <int FT, bool MHD, uint32_t RS>
__host__ __device__ constexpr uint32_t ws_row_bytes() {
    return row_streams<FT, MHD>() * RS * (uint32_t)sizeof(typename Ddf<FT>::T) + (MHD ? 6u * RS * 4u : 0u) + RS;
}

// Rows of up to 256 cells: three CTAs of up to 288 threads per SM (72 registers; FP16
// MHD rows of 256 cells then run 24 compute warps per SM instead of 16: 0.920 -> 0.845
// ms at 256^3 FP16S), except MHD with TRT, which spills at 72 registers.  Rows of up to
// 384 cells: two CTAs of up to 416 threads (78 registers), one for MHD with TRT.
template <uint32_t RS>
__host__ __device__ constexpr int ws_threads() { return RS == 384u ? 416 : 288; }
template <uint32_t RS, bool MHD, bool TRT>
__host__ __device__ constexpr int ws_min_ctas() { return RS == 384u ? ((MHD && TRT) ? 1 : 2) : ((MHD && TRT) ? 2 : 3); }
template <int FT, bool MHD, bool TRT, uint32_t RS>
__global__ void __launch_bounds__(ws_threads<RS>(), ws_min_ctas<RS, MHD, TRT>()) k_sc_rows_ws(const DevLbm L, const uint32_t odd_t, uint32_t* err) {
    using T = typename Ddf<FT>::T;
    constexpr uint32_t RB = ws_row_bytes<FT, MHD, RS>();
    constexpr uint32_t SB = RS * (uint32_t)sizeof(T);  // bytes per stream row
    constexpr uint32_t eb_off = row_streams<FT, MHD>() * SB, fl_off = eb_off + (MHD ? 6u * RS * 4u : 0u);
    extern __shared__ __align__(128) uint8_t rows_smem[];
    __shared__ __align__(8) uint64_t full[2], empty[2];
    __shared__ uint32_t fail_flag, issued;  // rows the producer has staged
    volatile uint32_t* fail = &fail_flag;
    const bool odd = odd_t != 0u;
    const uint32_t nx = L.nx, ny = L.ny, nz = L.nz, nrows = ny * nz, N = L.n;
    const uint32_t rb = nx * (uint32_t)sizeof(T);  // bytes of one stream's row in global memory
    const uint32_t nct = blockDim.x - 32u, ncw = nct / 32u;  // compute threads and warps
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1u);
        mbar_init(&full[1], 1u);
        mbar_init(&empty[0], ncw);
        mbar_init(&empty[1], ncw);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fail_flag = 0u;
        issued = 0u;
    }
    __syncthreads();
    const uint32_t my_rows = blockIdx.x < nrows ? (nrows - 1u - blockIdx.x) / gridDim.x + 1u : 0u;
    if (threadIdx.x >= nct) {
        if (threadIdx.x == nct) {
            auto for_streams = [&](uint32_t r, auto&& op) { for_row_streams<FT, MHD>(L, r, odd, op); };
            // row k of this CTA lives in buffer k & 1
            auto write_back = [&](uint32_t k) {
                const uint8_t* src = rows_smem + (k & 1u) * RB;
                for_streams(blockIdx.x + k * gridDim.x, [&](uint32_t st, T* g) { bulk_s2g(g, src + st * SB, rb); });
                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            };
            uint32_t k = 0;
            for (; k < my_rows; k++) {
                const uint32_t b = k & 1u, r = blockIdx.x + k * gridDim.x;
                if (k >= 2) {
                    // row k - 2 computed: copy it back, and wait until the copies have read the buffer
                    if (!mbar_wait_or_fail(&empty[b], ((k - 2) >> 1) & 1u, fail, L.wait_limit)) break;
                    if (*fail) break;
                    write_back(k - 2u);
                    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
                }
                if (*fail) break;
                uint8_t* dst = rows_smem + b * RB;
                const uint32_t y = r % ny, z = r / ny, own = (y + z * ny) * nx;
                mbar_expect_tx(&full[b], row_streams<FT, MHD>() * rb + (MHD ? 6u * nx * 4u : 0u) + ((nx + 15u) & ~15u));
                for_streams(r, [&](uint32_t st, T* g) { bulk_g2s(dst + st * SB, g, rb, &full[b]); });
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
                    if (!mbar_wait_or_fail(&empty[t & 1u], (t >> 1) & 1u, fail, L.wait_limit) || *fail) break;
                    write_back(t);
                }
            }
            asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
        }
        __syncwarp();
    } else {
        const uint32_t lane = threadIdx.x & 31u;
        for (uint32_t k = 0; k < my_rows; k++) {
            const uint32_t b = k & 1u, r = blockIdx.x + k * gridDim.x;
            const bool go = mbar_wait_or_fail(&full[b], (k >> 1) & 1u, fail, L.wait_limit) && *fail == 0u;
            if (go) {
                uint8_t* buf = rows_smem + b * RB;
                const uint32_t y = r % ny, z = r / ny;
                for (uint32_t x = threadIdx.x; x < nx; x += nct) {
                    const RowSrc<T, RS, true> S{buf, nx, x, x + 1u == nx ? 0u : x + 1u, x == 0u ? nx - 1u : x - 1u,
                                                 eb_off, fl_off};
                    sc_cell<19, FT, MHD, TRT, false, RowSrc<T, RS, true>, uint32_t>(L, x + (y + z * ny) * nx, odd, S);
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
        atomicExch(err, 1u);
    }
}

// the row kernels when the domain's rows can be copied as whole 16-byte-aligned
// streams and two buffers fit in shared memory; false: use k_stream_collide
template <int FT, bool MHD, bool TRT>
bool launch_sc_rows(const DevLbm& L, uint32_t o, uint32_t* err, cudaStream_t s) {
    // whole 16-byte rows, two buffers in shared memory, and 32-bit slot offsets (19 N < 2^32)
    const bool ws = L.nx <= WS_ROW;  // producer warp + one cell per thread and row
    const uint32_t rs = ws ? ws_stride(L.nx) : 0u;
    static_assert(2u * ws_row_bytes<ION_FP32, true, WS_ROW>() <= 200u * 1024u, "two row buffers of the widest form");
    const uint32_t smem = 2u * (rs == 128u   ? ws_row_bytes<FT, MHD, 128u>()
                                : rs == 256u ? ws_row_bytes<FT, MHD, 256u>()
                                : rs == 384u ? ws_row_bytes<FT, MHD, 384u>()
                                             : row_bytes<FT, MHD>(L.nx));
    if (L.nx % 16u || smem > 200u * 1024u || 19ull * L.n >= (1ull << 32)) return false;
    const uint32_t threads =
        ws ? (L.nx + 31u) / 32u * 32u + 32u : ((L.nx + ((L.nx + 255u) / 256u) - 1u) / ((L.nx + 255u) / 256u) + 31u) / 32u * 32u;
    auto kern = rs == 128u   ? k_sc_rows_ws<FT, MHD, TRT, 128u>
                : rs == 256u ? k_sc_rows_ws<FT, MHD, TRT, 256u>
                : rs == 384u ? k_sc_rows_ws<FT, MHD, TRT, 384u>
                             : k_sc_rows<FT, MHD, TRT>;
    // the shared-memory opt-in and the occupancy of the last shape, per instantiation
    // (handles may step on several host threads)
    static std::mutex mu;
    static bool attr[4] = {false, false, false, false};
    static int per_sm_of[4] = {0, 0, 0, 0};
    static uint32_t for_smem[4] = {0, 0, 0, 0}, for_threads[4] = {0, 0, 0, 0};
    const int v = (int)(rs / 128u);
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!attr[v]) {
            if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess)
                return false;
            attr[v] = true;
        }
        if (for_smem[v] != smem || for_threads[v] != threads) {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_of[v], kern, (int)threads, smem) != cudaSuccess ||
                per_sm_of[v] < 1)
                return false;
            for_smem[v] = smem;
            for_threads[v] = threads;
        }
        per_sm = per_sm_of[v];
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t rows = L.ny * L.nz;
    const uint32_t grid = std::min<uint32_t>(rows, (uint32_t)(per_sm * sms));
    kern<<<grid, threads, smem, s>>>(L, o, err);
    return true;
}

// ---------------------------------------------------------------------------
// initialize (sim_kernels.cl:760-832): equilibrium DDFs stored with parity 1
// ---------------------------------------------------------------------------
template <int Q, int FT, bool MHD, bool ECR = false>
__global__ void __launch_bounds__(256) k_initialize(const DevLbm L) {
    using V = VSet<Q>;
    using D = Ddf<FT>;
    using T = typename D::T;
    const uint32_t N = L.n;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        uint32_t x, y, z;
        cell_xyz(L, n, x, y, z);
        const Nbr nb(L, x, y, z);
        const NbV<V> j{nb};
        if ((L.flags[n] & F_BO) == F_S) {
            L.u[n] = 0.0f; L.u[(size_t)N + n] = 0.0f; L.u[2 * (size_t)N + n] = 0.0f;
            if constexpr (MHD) L.q[n] = 0.0f;
        }
        const float ux = L.u[n], uy = L.u[(size_t)N + n], uz = L.u[2 * (size_t)N + n];
        float feq[Q];
        equilibrium<V>(L.rho[n], ux, uy, uz, feq);
        ep_store<D, Q>((T*)L.fi, N, n, true, j, feq);
        if constexpr (MHD) {
            float aeq[7];
            // rho_e0 > 0 (finite-plasma start, no reference counterpart): ions at
            // Q + rho_e0 and electrons at rho_e0, the same net charge Q; rho_e0 = 0 is
            // the reference's start (electron gas at density 0, sim_kernels.cl:823)
            const float rq0 = L.rho_e0 != 0.0f ? L.q[n] + L.rho_e0 : L.q[n];
            adv_equilibrium(rq0, ux, uy, uz, aeq);
            const Nb7 j7{nb};
            ep_store<D, 7>((T*)L.fqi, N, n, true, j7, aeq);
#pragma unroll
            for (int c = 0; c < 3; c++) {
                L.b_dyn[(size_t)c * N + n] = L.b_stat[(size_t)c * N + n];
                L.e_dyn[(size_t)c * N + n] = L.e_stat[(size_t)c * N + n];
            }
            equilibrium<V>(L.rho_e0, ux, uy, uz, feq);
            ep_store<D, Q>((T*)L.ei, N, n, true, j, feq);
            if constexpr (ECR) {  // electron temperature DDFs (sim_kernels.cl:827-831)
                adv_equilibrium(L.et[n], ux, uy, uz, aeq);
                ep_store<D, 7>((T*)L.eti, N, n, true, j7, aeq);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// update_fields (sim_kernels.cl:834-859)
// ---------------------------------------------------------------------------
template <int Q, int FT>
__global__ void __launch_bounds__(256) k_update_fields(const DevLbm L, const uint32_t odd_t) {
    using V = VSet<Q>;
    using D = Ddf<FT>;
    using T = typename D::T;
    const uint32_t N = L.n;
    for (uint32_t n = blockIdx.x * blockDim.x + threadIdx.x; n < N; n += gridDim.x * blockDim.x) {
        if ((L.flags[n] & F_BO) == F_S) continue;
        uint32_t x, y, z;
        cell_xyz(L, n, x, y, z);
        const Nbr nb(L, x, y, z);
        const NbV<V> j{nb};
        float f[Q], rho, ux, uy, uz;
        ep_load<D, Q>((const T*)L.fi, N, n, odd_t != 0u, j, f);
        moments<V>(f, rho, ux, uy, uz);
        L.rho[n] = rho;
        L.u[n] = clampf(ux, -CS, CS);
        L.u[(size_t)N + n] = clampf(uy, -CS, CS);
        L.u[2 * (size_t)N + n] = clampf(uz, -CS, CS);
    }
}

// mode: 0 plain, 1 MAGNETO_HYDRO, 2 MAGNETO_HYDRO + SUBGRID_ECR
template <int QV, int FT>
void launch_sc(const DevLbm& L, int mode, bool trt, uint32_t o, unsigned g, uint32_t* err, cudaStream_t s) {
    if constexpr (QV == 19) {
        if (mode == 1 && (trt ? launch_sc_rows<FT, true, true>(L, o, err, s) : launch_sc_rows<FT, true, false>(L, o, err, s)))
            return;
        if (mode == 0 && (trt ? launch_sc_rows<FT, false, true>(L, o, err, s) : launch_sc_rows<FT, false, false>(L, o, err, s)))
            return;
    }
    if (mode == 2) {
        if (trt) k_stream_collide<QV, FT, true, true, true><<<g, 256, 0, s>>>(L, o);
        else k_stream_collide<QV, FT, true, false, true><<<g, 256, 0, s>>>(L, o);
    } else if (mode == 1) {
        if (trt) k_stream_collide<QV, FT, true, true><<<g, 256, 0, s>>>(L, o);
        else k_stream_collide<QV, FT, true, false><<<g, 256, 0, s>>>(L, o);
    } else {
        if (trt) k_stream_collide<QV, FT, false, true><<<g, 256, 0, s>>>(L, o);
        else k_stream_collide<QV, FT, false, false><<<g, 256, 0, s>>>(L, o);
    }
}
template <int QV, int FT>
void launch_init(const DevLbm& L, int mode, unsigned g, cudaStream_t s) {
    if (mode == 2) k_initialize<QV, FT, true, true><<<g, 256, 0, s>>>(L);
    else if (mode == 1) k_initialize<QV, FT, true><<<g, 256, 0, s>>>(L);
    else k_initialize<QV, FT, false><<<g, 256, 0, s>>>(L);
}

#define ION_DEFINE_LBM_DISPATCH(QV, NAME)                                                                     \
    void NAME##_stream_collide(const DevLbm& L, int ft, int mode, bool trt, uint64_t t, uint32_t* err,          \
                               cudaStream_t s) {                                                               \
        const unsigned g = grid_for(L.n, 256);                                                                 \
        const uint32_t o = (uint32_t)(t & 1u);                                                                 \
        if (ft == ION_FP32) launch_sc<QV, ION_FP32>(L, mode, trt, o, g, err, s);                               \
        else if (ft == ION_FP16S) launch_sc<QV, ION_FP16S>(L, mode, trt, o, g, err, s);                        \
        else launch_sc<QV, ION_FP16C>(L, mode, trt, o, g, err, s);                                             \
    }                                                                                                          \
    void NAME##_initialize(const DevLbm& L, int ft, int mode, cudaStream_t s) {                                \
        const unsigned g = grid_for(L.n, 256);                                                                 \
        if (ft == ION_FP32) launch_init<QV, ION_FP32>(L, mode, g, s);                                          \
        else if (ft == ION_FP16S) launch_init<QV, ION_FP16S>(L, mode, g, s);                                   \
        else launch_init<QV, ION_FP16C>(L, mode, g, s);                                                        \
    }                                                                                                          \
    void NAME##_update_fields(const DevLbm& L, int ft, uint64_t t, cudaStream_t s) {                           \
        const unsigned g = grid_for(L.n, 256);                                                                 \
        const uint32_t o = (uint32_t)(t & 1u);                                                                 \
        if (ft == ION_FP32) k_update_fields<QV, ION_FP32><<<g, 256, 0, s>>>(L, o);                             \
        else if (ft == ION_FP16S) k_update_fields<QV, ION_FP16S><<<g, 256, 0, s>>>(L, o);                      \
        else k_update_fields<QV, ION_FP16C><<<g, 256, 0, s>>>(L, o);                                           \
    }

}  // namespace ion
