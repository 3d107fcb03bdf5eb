/* Philox4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3", SC'11): 10 rounds of the
 * multiply-xor bijection with a Weyl key schedule (TEST INFRASTRUCTURE).
 * The kernels draw from this generator; the oracle (cmc_oracle.c) and the
 * driver of the reference's own step (refshim/refdrive.c) share this one
 * copy, pinned by the Random123 known-answer vectors in tests/golden. */
#ifndef CMC_PHILOX_H
#define CMC_PHILOX_H
#include <stdint.h>

static inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; ++round) {
        if (round > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

#endif
