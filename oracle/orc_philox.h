/*
 * orc_philox.h -- counter-based RNG used by the CPU oracle.
 *
 * TEST INFRASTRUCTURE (CPU oracle).  Only the test suite, the smoke check and
 * the CPU-baseline leg of bench.py use it.
 *
 * Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw, "Parallel
 * random numbers: as easy as 1, 2, 3" (SC'11): ten rounds of two 32x32->64
 * multiplies with the published multipliers and Weyl key increments.
 *
 * Stream layout (shared by the oracle, the reference shim and the GPU path):
 *   key     = (seed_lo32, seed_hi32 ^ history_hi32)
 *   counter = (draw >> 1, event, particle_id, history_lo32)
 *   draw d  = words (0,1) when d is even, words (2,3) when d is odd, joined as
 *             v = hi<<32 | lo and mapped to ((v >> 12) + 0.5) * 2^-52, an
 *             exact double in (0, 1).
 * Event 0 of particle 0 is the source sampling of a history; random-walk
 * iterations are events 1, 2, ...; a particle split off at a surface crossing
 * gets id = orc_child_id(parent, parent_event, k) for its k-th copy and starts
 * its own events at 1.  The reference's global LCG (Random.cpp:121-126) has no
 * per-history state, so it is replaced by this stream on both sides.
 */
#ifndef ORC_PHILOX_H
#define ORC_PHILOX_H
#include <stdint.h>

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2],
                                     uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline uint32_t orc_fmix32(uint32_t h)
{
    /* MurmurHash3 32-bit finaliser (public domain, Appleby). */
    h ^= h >> 16; h *= 0x85EBCA6Bu;
    h ^= h >> 13; h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return h;
}

static inline uint32_t orc_child_id(uint32_t parent, uint32_t event, uint32_t k)
{
    return orc_fmix32(parent * 0x9E3779B1u + orc_fmix32(event * 0x85EBCA77u + k));
}

typedef struct {
    uint64_t seed;
    uint64_t history;
    uint32_t id;
    uint32_t event;
    uint32_t draw;
} orc_rng;

static inline double orc_u01_from(uint32_t lo, uint32_t hi)
{
    uint64_t v = ((uint64_t)hi << 32) | lo;
    return ((double)(v >> 12) + 0.5) * (1.0 / 4503599627370496.0);  /* 2^-52 */
}

static inline double orc_urand(orc_rng *s)
{
    uint32_t ctr[4] = { s->draw >> 1, s->event, s->id, (uint32_t)s->history };
    uint32_t key[2] = { (uint32_t)s->seed,
                        (uint32_t)(s->seed >> 32) ^ (uint32_t)(s->history >> 32) };
    uint32_t o[4];
    orc_philox4x32_10(ctr, key, o);
    double u = (s->draw & 1u) ? orc_u01_from(o[2], o[3]) : orc_u01_from(o[0], o[1]);
    s->draw++;
    return u;
}

#endif /* ORC_PHILOX_H */
