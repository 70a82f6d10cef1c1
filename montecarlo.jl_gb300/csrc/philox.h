// Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11), usable from host and device.
//
// Stream layout shared by the CUDA path and the CPU oracle: draw number d of a
// chain with 64-bit seed s is philox(ctr = {d_lo, d_hi, 0, 0}, key = {s_lo, s_hi});
// the draw's 64-bit word is (out0 << 32) | out1.  Draws are consumed in the
// order of the reference's Julia RNG calls: field initialisation (n*M draws,
// site fastest, fields.jl:330 / :470), then per proposal an optional
// rand(1:3) (GHQ fields, fields.jl:565 / :629) and a rand() only when p <= 1
// (local_updates.jl:53).
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define DQMC_HD __host__ __device__ __forceinline__
#else
#define DQMC_HD inline
#endif

DQMC_HD uint64_t dqmc_philox_word(uint64_t key, uint64_t ctr) {
    uint32_t c0 = (uint32_t)ctr, c1 = (uint32_t)(ctr >> 32), c2 = 0u, c3 = 0u;
    uint32_t k0 = (uint32_t)key, k1 = (uint32_t)(key >> 32);
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return ((uint64_t)c0 << 32) | (uint64_t)c1;
}

// uniform double in [0, 1) from the top 53 bits
DQMC_HD double dqmc_word_to_uniform(uint64_t w) { return (double)(w >> 11) * 0x1.0p-53; }

// 0, 1 or 2 from the high part of w * 3 (rand(1:3) - 1)
DQMC_HD int dqmc_word_to_choice3(uint64_t w) {
#if defined(__CUDA_ARCH__)
    return (int)__umul64hi(w, 3ull);
#else
    return (int)(((unsigned __int128)w * 3u) >> 64);
#endif
}
