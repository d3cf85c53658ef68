// ion_device.cuh -- shared device-side definitions of the GB300 MHD-LBM path.
//
// Everything here is compiled with -fmad=false: a*b+c stays two IEEE
// roundings unless the code calls fmaf(), which is how the reference's
// kernels are written (IonSolver src/kernels/sim_kernels.cl).  Division and
// sqrt are the IEEE round-to-nearest ones (-prec-div=true -prec-sqrt=true).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include "ionsolver.h"

namespace ion {

// flag bits, IonSolver src/lbm/domain.rs:819-828
constexpr uint8_t F_S = 0x01, F_E = 0x02, F_C = 0x04, F_F = 0x08, F_M = 0x10, F_BO = 0x1F;

// lattice speed of sound c = 1/sqrt(3) as the literal DEF_C (domain.rs:807)
constexpr float CS = 0.57735027f;
constexpr float THIRD = 0.33333334f;  // literal of sim_kernels.cl:369-375

// ---------------------------------------------------------------------------
// Velocity sets (directions in +/- pairs; order of sim_kernels.cl:326-347).
// ---------------------------------------------------------------------------
template <int Q> struct VSet;

template <> struct VSet<19> {
    static constexpr int q = 19, dims = 3;
    __host__ __device__ static constexpr int c(int i, int a) {
        constexpr int8_t t[19][3] = {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1},{1,1,0},{-1,-1,0},
                                     {1,0,1},{-1,0,-1},{0,1,1},{0,-1,-1},{1,-1,0},{-1,1,0},{1,0,-1},{-1,0,1},
                                     {0,1,-1},{0,-1,1}};
        return t[i][a];
    }
    __host__ __device__ static constexpr int wc(int i) { return i == 0 ? 0 : (i < 7 ? 1 : 2); }
    // DEF_W0/WS/WE of get_device_defines (domain.rs:763-765)
    __host__ __device__ static constexpr float w(int k) { return k == 0 ? (1.0f / 3.0f) : k == 1 ? (1.0f / 18.0f) : (1.0f / 36.0f); }
};

template <> struct VSet<15> {
    static constexpr int q = 15, dims = 3;
    __host__ __device__ static constexpr int c(int i, int a) {
        constexpr int8_t t[15][3] = {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{0,0,1},{0,0,-1},{1,1,1},{-1,-1,-1},
                                     {1,1,-1},{-1,-1,1},{1,-1,1},{-1,1,-1},{-1,1,1},{1,-1,-1}};
        return t[i][a];
    }
    __host__ __device__ static constexpr int wc(int i) { return i == 0 ? 0 : (i < 7 ? 1 : 2); }
    __host__ __device__ static constexpr float w(int k) { return k == 0 ? (1.0f / 4.5f) : k == 1 ? (1.0f / 9.0f) : (1.0f / 72.0f); }
};

template <> struct VSet<9> {
    static constexpr int q = 9, dims = 2;
    __host__ __device__ static constexpr int c(int i, int a) {
        constexpr int8_t t[9][3] = {{0,0,0},{1,0,0},{-1,0,0},{0,1,0},{0,-1,0},{1,1,0},{-1,-1,0},{1,-1,0},{-1,1,0}};
        return t[i][a];
    }
    __host__ __device__ static constexpr int wc(int i) { return i == 0 ? 0 : (i < 5 ? 1 : 2); }
    __host__ __device__ static constexpr float w(int k) { return k == 0 ? (1.0f / 2.25f) : k == 1 ? (1.0f / 9.0f) : (1.0f / 36.0f); }
};

// ---------------------------------------------------------------------------
// 32-bit unsigned division by a runtime-invariant divisor (Granlund &
// Montgomery, "Division by invariant integers using multiplication", 1994,
// round-up variant with a 33-bit intermediate): q = (umulhi(n,m) + n) >> l.
// ---------------------------------------------------------------------------
struct FastDiv {
    uint32_t d, m, l;
    // trivial, so DevLbm can live in __shared__; a zero-initialised FastDiv
    // (m = 0, l = 0) returns n, i.e. divides by 1
    FastDiv() = default;
    explicit FastDiv(uint32_t div) : d(div) {
        l = 0;
        while ((1ull << l) < div) l++;
        m = (uint32_t)((((1ull << 32) * ((1ull << l) - div)) / div) + 1ull);
    }
    __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
        const uint32_t t = __umulhi(n, m);
#else
        const uint32_t t = (uint32_t)(((uint64_t)n * m) >> 32);
#endif
        return (uint32_t)(((uint64_t)t + n) >> l);
    }
};

// ---------------------------------------------------------------------------
// DDF storage codecs.
//   FP32 : plain float.
//   FP16S: IEEE binary16 of x*2^15, round to nearest even
//          (vstore_half_rte / vload_half, domain.rs:773-776).
//   FP16C: the reference's 1-4-11 format (sim_kernels.cl:79-90): the float's
//          bit pattern plus 2^11, 4 exponent bits (bias 15), 11 mantissa bits.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t fbits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u; __builtin_memcpy(&u, &f, 4); return u;
#endif
}
__host__ __device__ __forceinline__ float bitsf(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f; __builtin_memcpy(&f, &u, 4); return f;
#endif
}

// v >> s with shifts of 32 or more giving 0 (PTX shr clamps the shift amount)
__host__ __device__ __forceinline__ uint32_t shr_clamped(uint32_t v, uint32_t s) {
#ifdef __CUDA_ARCH__
    uint32_t r;
    asm("shr.b32 %0, %1, %2;" : "=r"(r) : "r"(v), "r"(s));
    return r;
#else
    return s >= 32u ? 0u : v >> s;
#endif
}

// A NaN is encoded as the canonical quiet NaN 0x7FFFFFFF would be (the bit
// pattern NVIDIA hardware gives every NaN result), so the stored value does
// not depend on where a NaN came from.  The reference's MHD step produces
// NaNs by itself: its electron density starts at 0 (sim_kernels.cl:823) and
// reaches exactly 0 again, so u_e = 0/0 (sim_kernels.cl:230-232).
__host__ __device__ __forceinline__ uint16_t fp16c_encode(float x) {
    const uint32_t xb = fbits(x);
    const uint32_t b = (((xb & 0x7FFFFFFFu) > 0x7F800000u) ? 0x7FFFFFFFu : xb) + 0x800u;
    const uint32_t e = (b >> 23) & 0xFFu;
    // both candidates, then a select (no divergent branch when a warp mixes normal and
    // subnormal results).  Normal (e > 112): the exponent rebiased by -112 into 4 bits
    // next to the top 11 mantissa bits, i.e. (b >> 12) - (112 << 11) in 15 bits.
    // Subnormal: the 24-bit significand shifted by 124 - e, then halved with rounding;
    // for e <= 100 the shift is 24 or more and the result 0, as the reference's
    // (e > 100) factor gives.  Equal to the reference's expression for all 2^32 inputs.
    const uint32_t nrm = ((b >> 12) - (112u << 11)) & 0x7FFFu;
    const uint32_t sub = (shr_clamped((b & 0x007FFFFFu) + 0x007FF800u, 124u - e) + 1u) >> 1;
    return (uint16_t)(((b >> 16) & 0x8000u) | (e > 112u ? nrm : sub));
}
__host__ __device__ __forceinline__ float fp16c_decode(uint16_t x) {
    const uint32_t mag = x & 0x7FFFu, sign = (uint32_t)(x & 0x8000u) << 16;
    // exponent field > 0: sign | (e + 112) << 23 | m << 12, one shift and one add.
    // Exponent field 0: the same bits read as a float are 2^-15 + m 2^-26, so
    // 2 (that) - 2^-14 = m 2^-25 exactly (one FMA, no integer conversion), which is the
    // normalised float the reference's leading-zero count builds.  Equal to the
    // reference's decoder for all 2^16 inputs.
    const uint32_t nrm = (mag << 12) + (112u << 23);
    const uint32_t sub = fbits(fmaf(bitsf(nrm), 2.0f, -6.103515625e-05f));
    return bitsf(sign | (mag >= 0x0800u ? nrm : sub));
}

// Packed FP32 pairs (PTX add/sub/mul/fma .f32x2, sm_100 and later): one
// instruction does the same IEEE round-to-nearest operation on the two halves
// of a 64-bit register (each instruction checked against the scalar one on the
// device), so two cells advance with half the issue slots.  A pair lives in a
// 64-bit integer (low half = first cell) from load to store, so no packing moves
// are needed between the instructions.  One caveat, measured on GB300 with CUDA
// 13.0: ptxas contracts a packed multiply that feeds a packed add into a packed
// FMA even under --fmad=false (which it honours for scalar code), also when the
// multiply is written as an FMA with a -0 addend or as volatile asm.  So packed
// code is only bit-identical to the scalar form where no inexact product feeds an
// addition; the FAST field, which uses these, is an approximation anyway.
using P2 = unsigned long long;
__device__ __forceinline__ P2 pk(float lo, float hi) {
    P2 r;
    asm("mov.b64 %0, {%1,%2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
// (the unpack writes both halves; the unused one draws warning 550)
#pragma nv_diag_suppress 550
__device__ __forceinline__ float lo32(P2 v) {
    float a, b;
    asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return a;
}
__device__ __forceinline__ float hi32(P2 v) {
    float a, b;
    asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
    return b;
}
#pragma nv_diag_default 550
__device__ __forceinline__ float half(P2 v, bool hi) { return hi ? hi32(v) : lo32(v); }
__device__ __forceinline__ void set_half(P2& v, bool hi, float x) { v = hi ? pk(lo32(v), x) : pk(x, hi32(v)); }
__device__ __forceinline__ P2 add2(P2 a, P2 b) {
    P2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ P2 mul2(P2 a, P2 b) {
    P2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ P2 fma2(P2 a, P2 b, P2 c) {
    P2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ P2 sub2(P2 a, P2 b) {
    P2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// shared memory, mbarriers and bulk asynchronous copies (cp.async.bulk, completion
// counted in bytes on an mbarrier)
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

// Polls before a wait for staged data gives up (the default of DevLbm::wait_limit).
// A wait that gives up records an error and skips its tile; the copies still in
// flight are then waited for with this full limit before the block exits.
constexpr uint32_t WAIT_LIMIT = 1u << 24;

template <int FT> struct Ddf;
template <> struct Ddf<ION_FP32> {
    using T = float;
    __device__ __forceinline__ static float dec(float v) { return v; }
    __device__ __forceinline__ static float enc(float x) { return x; }
    __device__ __forceinline__ static float ld(const float* p, size_t i) { return p[i]; }
    __device__ __forceinline__ static void st(float* p, size_t i, float x) { p[i] = x; }
};
template <> struct Ddf<ION_FP16S> {
    using T = uint16_t;
    __device__ __forceinline__ static float dec(uint16_t v) { return __half2float(__ushort_as_half(v)) * 3.0517578E-5f; }
    __device__ __forceinline__ static uint16_t enc(float x) { return __half_as_ushort(__float2half_rn(x * 32768.0f)); }
    __device__ __forceinline__ static float ld(const uint16_t* p, size_t i) { return dec(p[i]); }
    __device__ __forceinline__ static void st(uint16_t* p, size_t i, float x) { p[i] = enc(x); }
};
template <> struct Ddf<ION_FP16C> {
    using T = uint16_t;
    __device__ __forceinline__ static float dec(uint16_t v) { return fp16c_decode(v); }
    __device__ __forceinline__ static uint16_t enc(float x) { return fp16c_encode(x); }
    __device__ __forceinline__ static float ld(const uint16_t* p, size_t i) { return dec(p[i]); }
    __device__ __forceinline__ static void st(uint16_t* p, size_t i, float x) { p[i] = enc(x); }
};

// x / b rounded to nearest, for finite b > 0, from y = RN(1/b) (__frcp_rn):
// q0 = RN(x y); the residual r = x - q b is exact under an FMA when q is
// within a few ulps of x/b; q1 = RN(q0 + r0 y) is within half an ulp plus a
// tiny term, and Markstein's theorem (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34(1), 1990; also Muller et al., Handbook of Floating-Point
// Arithmetic, ch. 4) makes q2 = RN(q1 + r1 y) the correctly rounded quotient
// when y = RN(1/b) and q1 is within one ulp -- barring overflow, underflow and
// subnormals, which the E/B sums never reach (|x| <= 2^13, 2^-3 <= b <= 2^40,
// and x = 0 gives +0 as x / b does for x = +0).  Three quotients by the same b
// then cost one reciprocal and 5 FMA-pipe operations each instead of three
// full divisions.  ion_check_shared_division compares it bit for bit with the
// IEEE division on the device.
__device__ __forceinline__ float div_rn_shared(float x, float b, float y) {
    float q = x * y;
    float r = fmaf(-q, b, x);
    q = fmaf(r, y, q);
    r = fmaf(-q, b, x);
    return fmaf(r, y, q);
}

// ---------------------------------------------------------------------------
// Device view of one domain (all pointers are device memory).
// ---------------------------------------------------------------------------
struct DevLbm {
    uint32_t nx, ny, nz;
    uint32_t n;            // cells (< 2^32, as the reference's uint n)
    FastDiv dx, dxy;       // divisions by nx and nx*ny
    void* fi;              // [q][N]
    float* rho;            // [N]
    float* u;              // [3][N]
    uint8_t* flags;        // [N]
    float* F;              // [3][N] or null
    float *e_stat, *b_stat, *e_dyn, *b_dyn;  // [3][N]
    void* fqi;             // [7][N]
    void* ei;              // [q][N]
    float* q;              // [N]
    float* qu_lod;         // [n_lod][4]
    float* lod_cell;       // scratch [3][N]: u*ils per cell for the LOD sums
    float4* lod_pos;       // [n_lod_own] LOD bin centres
    float w, ke, kmu, kmu0, kkge, wq;
    float fx, fy, fz;
    uint32_t depth, nd, n_lod_own, n_bins, first_src;
    uint32_t bsx, bsy, bsz;      // LOD bin extent in cells
    uint32_t near_x, near_y, near_z;  // near-field block extent
    float ils;
    float* e_var;          // [3][N] SUBGRID_ECR oscillating field (or null)
    void* eti;             // [7][N] SUBGRID_ECR electron-temperature DDFs (or null)
    float* et;             // [N]    SUBGRID_ECR electron temperature (or null)
    float kkbme, keabs;    // DEF_KKBME, DEF_KEABS
    float rho_e0;          // background electron density of the finite-plasma start (0: reference start)
    uint32_t wait_limit;   // polls before a bounded wait gives up (WAIT_LIMIT unless lowered)
    uint8_t ext_eq, ext_vf, ext_ff, ext_mhd, update_fields, trt;
};

__device__ __forceinline__ void cell_xyz(const DevLbm& L, uint32_t n, uint32_t& x, uint32_t& y, uint32_t& z) {
    z = L.dxy.div(n);
    const uint32_t r = n - z * L.nx * L.ny;
    y = L.dx.div(r);
    x = r - y * L.nx;
}

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

}  // namespace ion
