// tcgen05.cuh -- small helpers for the 5th-generation tensor-core path on sm_103a
// (shared-memory matrix descriptors, instruction descriptors, bounded mbarrier
// waits), used by the network convolution and the tensor-core field update.
#pragma once
#include <cstdint>

namespace ion {
namespace tc {

__device__ __forceinline__ uint32_t saddr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start >> 4 [0,14), LBO >> 4 [16,30), SBO >> 4 [32,46),
// version 1 [46,48), base offset 0, layout SWIZZLE_NONE (0) [61,64).  For the no-swizzle
// K-major layout a core matrix is 8 rows x 16 bytes stored contiguously; LBO is the byte
// distance between core matrices adjacent in K, SBO between adjacent 8-row groups.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16 / kind::tf32: D F32 [4,6) = 1, A type [7,10), B type
// [10,13) (F16 0, BF16 1, TF32 2; A and B of the same type), A and B K-major (bits 15, 16
// = 0), N >> 3 [17,23), M >> 4 [24,29)
enum : uint32_t { TYPE_BF16 = 1u, TYPE_TF32 = 2u };
__host__ __device__ constexpr uint32_t idesc(uint32_t m, uint32_t n, uint32_t type) {
    return (1u << 4) | (type << 7) | (type << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n) { return idesc(m, n, TYPE_BF16); }

// waits for the phase of the given parity of an mbarrier; false after 2^24 polls
__device__ __forceinline__ bool wait(uint64_t* bar, uint32_t parity) {
    for (uint32_t i = 0; i < (1u << 24); i++) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(done) : "r"(saddr(bar)), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

}  // namespace tc
}  // namespace ion
