// rng.cuh — Philox4x32-10 counter-based generator (Salmon, Moraes, Dror,
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11), used so that
// every (replica, tile, window, event) draw is reproducible independently of
// launch order.  The reference draws from one serial ran3 stream
// (mulskips-source/mcevent/random.f:22-69), which has no parallel form.
#pragma once
#include <stdint.h>

namespace mks {

struct U4 {
    uint32_t x, y, z, w;
};

__host__ __device__ __forceinline__ void philox_mulhilo(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo)
{
    uint64_t p = (uint64_t)a * (uint64_t)b;
    hi = (uint32_t)(p >> 32);
    lo = (uint32_t)p;
}

__host__ __device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        philox_mulhilo(M0, c.x, hi0, lo0);
        philox_mulhilo(M1, c.z, hi1, lo1);
        U4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// uniform in (0, 1): 24 random bits, offset by half an ulp
__host__ __device__ __forceinline__ float u01(uint32_t v)
{
    return ((float)(v >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

}  // namespace mks
