/*
 * bamf_philox.h - the per-chain uniform stream shared by the CUDA sampler,
 * the CPU oracle and the reference-sampler driver.
 *
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11): a counter-based generator, so uniform number i
 * of chain r can be computed without generating 0..i-1.  That is what lets a
 * GPU warp generate 32 blocks of the stream in parallel while the CPU oracle
 * walks it one value at a time, with the same values on both sides.
 *
 * Stream definition (the parity contract):
 *   key     = (seed, chain_id)
 *   block b = Philox4x32_10(counter = (b, 0, 0, 0), key)   -> 4 words
 *   value i = block(i >> 2).word[i & 3] >> 1                -> 31-bit int k
 *
 * The reference draws uniforms as (float)rand() / ((float)RAND_MAX + 1)
 * (source/c/LibRJMCMCreturn.hpp:17) with glibc's RAND_MAX = 2^31 - 1, so a
 * 31-bit k in [0, 2^31) stands in for rand(); bamf_u31_to_float() then does
 * the reference's exact float conversion: (float)k rounds to 24 bits (it can
 * round up to 2^31) and the divisor (float)RAND_MAX + 1 is exactly 2^31, so
 * urand lies in [0, 1] inclusive, as in the reference.
 *
 * Usable from C, C++ and CUDA device code.
 */
#ifndef BAMF_PHILOX_H
#define BAMF_PHILOX_H

#include <stdint.h>

#if defined(__CUDACC__)
#define BAMF_PHILOX_HD __host__ __device__ static inline
#else
#define BAMF_PHILOX_HD static inline
#endif

#define BAMF_PHILOX_M0 0xD2511F53u
#define BAMF_PHILOX_M1 0xCD9E8D57u
#define BAMF_PHILOX_W0 0x9E3779B9u
#define BAMF_PHILOX_W1 0xBB67AE85u

typedef struct { uint32_t v[4]; } bamf_philox_block;

BAMF_PHILOX_HD void bamf_mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo)
{
#if defined(__CUDA_ARCH__)
    *hi = __umulhi(a, b);
    *lo = a * b;
#else
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
#endif
}

/* Ten Philox rounds on counter c with key (k0, k1). */
BAMF_PHILOX_HD bamf_philox_block bamf_philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2,
                                                    uint32_t c3, uint32_t k0, uint32_t k1)
{
    bamf_philox_block r;
    for (int round = 0; round < 10; ++round) {
        uint32_t hi0, lo0, hi1, lo1;
        bamf_mulhilo32(BAMF_PHILOX_M0, c0, &hi0, &lo0);
        bamf_mulhilo32(BAMF_PHILOX_M1, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += BAMF_PHILOX_W0;
        k1 += BAMF_PHILOX_W1;
    }
    r.v[0] = c0; r.v[1] = c1; r.v[2] = c2; r.v[3] = c3;
    return r;
}

/* 31-bit value i of the stream keyed by (seed, chain). */
BAMF_PHILOX_HD uint32_t bamf_stream_u31(uint32_t seed, uint32_t chain, uint32_t i)
{
    bamf_philox_block b = bamf_philox4x32_10(i >> 2, 0u, 0u, 0u, seed, chain);
    return b.v[i & 3u] >> 1;
}

/* The reference's urand() applied to a 31-bit draw: (float)k / 2^31. */
BAMF_PHILOX_HD float bamf_u31_to_float(uint32_t k)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(__int2float_rn((int)k), 4.656612873077392578125e-10f);
#else
    return (float)(int)k * 4.656612873077392578125e-10f;
#endif
}

#endif /* BAMF_PHILOX_H */
