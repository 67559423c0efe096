/*
 * mg_philox.h - counter-based random numbers for the batched HMC moves (mg_hmc_batch).
 *
 * Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw, "Parallel random numbers:
 * as easy as 1, 2, 3" (SC'11): ten rounds of two 32x32->64-bit multiplications with a
 * Weyl-sequence key schedule. A draw is a pure function of (key, counter), so every
 * replica, move and atom has its own stream and the engine, the CPU checker and any
 * caller reproduce the same numbers without shared state. Header-only C99, also
 * compiled as CUDA device code.
 *
 * Streams used by mg_hmc_batch: key = (seed low 32 bits, seed high 32 bits), counter =
 * (atom index in its replica, move index, purpose, replica index); purpose 0 and 1 give
 * the atom's three Maxwell-Boltzmann velocity components (Box-Muller), purpose 2 with
 * atom index 0 the Metropolis uniform.
 */
#ifndef MG_PHILOX_H_
#define MG_PHILOX_H_

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define MG_HD __host__ __device__ __forceinline__
#else
#define MG_HD static inline
#endif

MG_HD void mg_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3], k0 = key[0], k1 = key[1];
#if defined(__CUDACC__)
#pragma unroll
#endif
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * x0, p1 = (uint64_t)0xCD9E8D57u * x2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1;
        x0 = n0;
        x1 = (uint32_t)p1;
        x2 = n2;
        x3 = (uint32_t)p0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = x0;
    out[1] = x1;
    out[2] = x2;
    out[3] = x3;
}

/* uniform in (0, 1] from two 32-bit words (53 significant bits) */
MG_HD double mg_u01(uint32_t hi, uint32_t lo) {
    const uint64_t m = (((uint64_t)hi << 32) | lo) >> 11;
    return ((double)m + 1.0) * 1.1102230246251565e-16; /* 2^-53 */
}

/* two standard normal deviates (Box-Muller) from one draw */
MG_HD void mg_gauss2(const uint32_t w[4], double *g0, double *g1) {
    const double u1 = mg_u01(w[0], w[1]), u2 = mg_u01(w[2], w[3]);
    const double r = sqrt(-2.0 * log(u1));
    const double t = 6.283185307179586 * u2;
    *g0 = r * cos(t);
    *g1 = r * sin(t);
}

#endif /* MG_PHILOX_H_ */
