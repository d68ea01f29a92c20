// Counter-based random numbers for the GPU samplers: Philox4x32-10 (Salmon,
// Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC 2011)
// with the published round multipliers and Weyl key increments, and the
// conversions of its 32-bit outputs to uniform doubles.
#pragma once
#include <cstdint>

namespace rfba {

// Philox4x32 round function and key schedule (published constants).
struct Philox {
    static __device__ __forceinline__ void round(uint32_t c[4], const uint32_t k[2]) {
        const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
        const uint32_t hi0 = __umulhi(M0, c[0]), lo0 = M0 * c[0];
        const uint32_t hi1 = __umulhi(M1, c[2]), lo1 = M1 * c[2];
        const uint32_t n0 = hi1 ^ c[1] ^ k[0], n1 = lo1, n2 = hi0 ^ c[3] ^ k[1], n3 = lo0;
        c[0] = n0;
        c[1] = n1;
        c[2] = n2;
        c[3] = n3;
    }
    static __device__ __forceinline__ void gen(uint32_t c[4], uint32_t k0, uint32_t k1) {
        uint32_t k[2] = {k0, k1};
#pragma unroll
        for (int r = 0; r < 10; ++r) {
            round(c, k);
            k[0] += 0x9E3779B9u;
            k[1] += 0xBB67AE85u;
        }
    }
};

__device__ __forceinline__ double u53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);  // [0, 1)
}
__device__ __forceinline__ double u32(uint32_t a) { return ((double)a + 0.5) * (1.0 / 4294967296.0); }  // (0, 1)

}  // namespace rfba
