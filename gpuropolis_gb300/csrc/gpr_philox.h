/*
 * gpr_philox.h -- counter-based random stream used by the "philox" RNG mode.
 *
 * Philox4x32 with 10 rounds, the published generator of Salmon, Moraes, Dror
 * and Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11): two 32x32
 * multiply-hi/lo S-boxes per round, Weyl-sequence key schedule.
 *
 * Stream layout.  A chain's stream inside one block of MH steps is keyed by
 * (block seed, chain index); draw j of that stream is word (j mod 4) of
 * Philox(counter = (j / 4, 0, 0, 0)), shifted right by one so that, like the
 * reference's LCG (main.cu:210-216), every draw is a non-negative 31-bit int.
 * Jumping to draw j is O(1), which is what lets the kernel hand the constant
 * proposals of one chain to 32 lanes at once.
 */
#ifndef GPR_PHILOX_H
#define GPR_PHILOX_H

#include <stdint.h>

#ifndef GPR_HD
#if defined(__CUDACC__)
#define GPR_HD __host__ __device__ __forceinline__
#else
#define GPR_HD static inline
#endif
#endif

GPR_HD void gpr_philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)M0 * c[0];
        uint64_t p1 = (uint64_t)M1 * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0;
        uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
        k0 += W0; k1 += W1;
    }
}

/* Draw number j (0-based) of the stream keyed by (seed, chain). */
GPR_HD int gpr_philox_draw(uint32_t seed, uint32_t chain, uint32_t j) {
    uint32_t c[4] = {j >> 2, 0u, 0u, 0u};
    gpr_philox4x32_10(c, seed, chain);
    return (int)(c[j & 3u] >> 1);
}

/* Sequential view of the same stream, for code written draw-after-draw. */
typedef struct {
    uint32_t seed, chain, next;
} gpr_philox_stream;

GPR_HD void gpr_philox_stream_init(gpr_philox_stream* s, uint32_t seed, uint32_t chain) {
    s->seed = seed; s->chain = chain; s->next = 0u;
}

GPR_HD int gpr_philox_stream_next(gpr_philox_stream* s) {
    return gpr_philox_draw(s->seed, s->chain, s->next++);
}

#endif /* GPR_PHILOX_H */
