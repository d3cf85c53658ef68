// ion_ref_compat.hpp -- test infrastructure (oracle), not product code.
//
// A small OpenCL C -> C++20 compatibility layer so that the reference's own
// kernel text (IonSolver src/kernels/sim_kernels.cl, the part after the
// `EndTempDefines%` marker, exactly what src/opencl.rs:67-75 hands to the
// OpenCL compiler) compiles as ordinary C++ and runs on host cores.
//
// Semantics chosen for the OpenCL builtins the kernels use:
//   - float3/uint3/int3: component-wise operators; a scalar converts to a
//     vector by broadcast (OpenCL C 6.3 "usual arithmetic conversions").
//   - dot/cross/length: the textbook formulas evaluated left to right in
//     IEEE single precision (the OpenCL spec leaves the order open; a GPU
//     OpenCL compiler may fuse these, which this oracle does not).
//   - clamp(x,lo,hi) = fmin(fmax(x,lo),hi) (OpenCL C 6.13.4).
//   - vload_half / vstore_half_rte: exact binary16 -> binary32 and
//     round-to-nearest-even binary32 -> binary16 (IEEE 754-2008 3.4, 4.3.1),
//     written here from the format definition.
//   - atomic_xchg on float: a sequentially consistent exchange of the bits.
//   - get_global_id(0): a thread-local work-item index set by the host program.
//   - printf inside kernels is compiled out.
// The whole translation unit is compiled with -ffp-contract=off so that no
// a*b+c is fused unless the kernel text itself calls fma().
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdlib>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

namespace ionref {

typedef uint8_t uchar;
typedef uint16_t ushort;
typedef uint32_t uint;
typedef uint64_t ulong;
typedef uint16_t half;  // storage type behind vload_half / vstore_half_rte

extern thread_local uint64_t g_gid;
inline uint64_t get_global_id(int) { return g_gid; }

struct float3 {
    float x, y, z;
    float3() : x(0.0f), y(0.0f), z(0.0f) {}
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
    float3(float s) : x(s), y(s), z(s) {}
    float3& operator+=(const float3& o) { x = x + o.x; y = y + o.y; z = z + o.z; return *this; }
    float3& operator-=(const float3& o) { x = x - o.x; y = y - o.y; z = z - o.z; return *this; }
};
inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(float3 a, float3 b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator*(float s, float3 b) { return float3(s * b.x, s * b.y, s * b.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator/(float3 a, float s) { return float3(a.x / s, a.y / s, a.z / s); }
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }

struct uint3 {
    uint x, y, z;
    uint3() : x(0u), y(0u), z(0u) {}
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};
inline uint3 operator+(uint3 a, uint3 b) { return uint3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline uint3 operator-(uint3 a, uint3 b) { return uint3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline uint3 operator*(uint3 a, uint s) { return uint3(a.x * s, a.y * s, a.z * s); }

struct int3 {
    int x, y, z;
    int3() : x(0), y(0), z(0) {}
    int3(int a, int b, int c) : x(a), y(b), z(c) {}
};

inline float3 convert_float3(uint3 v) { return float3((float)v.x, (float)v.y, (float)v.z); }

// OpenCL C's float pi (the value of M_PI_F rounded to float)
#define M_PI_F 3.14159274101257324219f
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 cross(float3 a, float3 b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float length(float3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

inline float clamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }
inline int clamp(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }
template <class T> inline T min(T a, T b) { return b < a ? b : a; }
template <class T> inline T max(T a, T b) { return a < b ? b : a; }
using std::abs;
using std::fma;
using std::sqrt;

inline uint as_uint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline float as_float(uint u) { float f; std::memcpy(&f, &u, 4); return f; }

// binary16 -> binary32, exact.
inline float half_bits_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t e = (h >> 10) & 0x1Fu;
    const uint32_t m = h & 0x3FFu;
    if (e == 0u) {  // zero or subnormal: m * 2^-24
        const float v = std::ldexp((float)m, -24);
        return sign ? -v : v;
    }
    if (e == 31u) return as_float(sign | 0x7F800000u | (m << 13) | (m ? 0x00400000u : 0u));
    return as_float(sign | ((e + 112u) << 23) | (m << 13));
}
// binary32 -> binary16, round to nearest, ties to even; overflow -> inf.
inline uint16_t float_to_half_bits_rte(float f) {
    const uint32_t x = as_uint(f);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7FFFFFFFu;
    if (ax >= 0x7F800000u) return (uint16_t)(sign | (ax > 0x7F800000u ? (0x7E00u | ((ax >> 13) & 0x3FFu)) : 0x7C00u));
    if (ax >= 0x477FF000u) return (uint16_t)(sign | 0x7C00u);  // >= 65520 rounds to inf
    if (ax >= 0x38800000u) {                                   // normal binary16
        uint32_t r = ax - 0x38000000u;
        r = r + 0x0FFFu + ((r >> 13) & 1u);
        return (uint16_t)(sign | (r >> 13));
    }
    if (ax <= 0x33000000u) return (uint16_t)sign;  // <= 2^-25 rounds to zero
    const uint32_t e = ax >> 23;
    const uint32_t m = (ax & 0x7FFFFFu) | 0x800000u;
    const uint32_t s = 126u - e;  // 14..24
    uint32_t res = m >> s;
    const uint32_t rem = m & ((1u << s) - 1u);
    const uint32_t halfway = 1u << (s - 1u);
    if (rem > halfway || (rem == halfway && (res & 1u))) res++;
    return (uint16_t)(sign | res);
}
inline float vload_half(size_t offset, const half* p) { return half_bits_to_float(p[offset]); }
inline void vstore_half_rte(float data, size_t offset, half* p) { p[offset] = float_to_half_bits_rte(data); }

inline float atomic_xchg(volatile float* p, float v) {
    uint32_t nv;
    std::memcpy(&nv, &v, 4);
    uint32_t old = __atomic_exchange_n((volatile uint32_t*)p, nv, __ATOMIC_SEQ_CST);
    float o;
    std::memcpy(&o, &old, 4);
    return o;
}

}  // namespace ionref

