// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11), usable from host C++ and device code.
//
// Counter layout used throughout the library (one call gives four 32-bit words):
//   c0 = logical box index of the site (x + E*(y + E*z))  or another per-item index
//   c1 = low 32 bits of the chain's sweep number
//   c2 = high 28 bits of the sweep number | stream selector << 28
//   c3 = chain index
//   key = the context seed (low, high 32 bits)
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define NMMC_HD __host__ __device__ __forceinline__
#else
#define NMMC_HD inline
#endif

enum : uint32_t {
    NMMC_STREAM_SWEEP = 0u,   // Metropolis proposals and acceptance uniforms
    NMMC_STREAM_INIT = 1u,    // random starting spins (field_type::all_rand)
    NMMC_STREAM_MASK = 2u,    // Weibull shape test, one uniform per box site
    NMMC_STREAM_SIZE = 3u,    // log-normal particle sizes
    NMMC_STREAM_NOISE = 4u    // generator noise inputs
};

struct nmmc_u4 { uint32_t x, y, z, w; };

NMMC_HD nmmc_u4 nmmc_philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                            uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#if defined(__CUDA_ARCH__)
        uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
        uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
#else
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return nmmc_u4{c0, c1, c2, c3};
}

// Uniform float in (0,1) from the top 23 bits: (k + 1/2) 2^-23, exact in FP32. On the device
// it is built from bits: (1 + k 2^-23) - (1 - 2^-24) is exact (Sterbenz) and equals the same value.
NMMC_HD float nmmc_u01f(uint32_t r) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(0x3f800000u | (r >> 9)) - 0.99999994f;
#else
    return ((float)(r >> 9) + 0.5f) * (1.0f / 8388608.0f);
#endif
}
// Uniform double in [0,1) from 32 bits.
NMMC_HD double nmmc_u01d(uint32_t r) { return (double)r * (1.0 / 4294967296.0); }
