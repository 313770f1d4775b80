/*
 * ORACLE (test infrastructure only; never linked into the product library).
 *
 * Counter-based Philox4x32-10 generator, restated from the published algorithm
 * (J. K. Salmon, M. A. Moraes, R. O. Dror, D. E. Shaw, "Parallel random numbers:
 * as easy as 1, 2, 3", SC'11): two 32x32->64 multiplies per round with the
 * multipliers 0xD2511F53 / 0xCD9E8D57 and a Weyl key schedule 0x9E3779B9 /
 * 0xBB67AE85, ten rounds.
 *
 * The reference (Merzbild.jl) draws every random number from one sequential
 * Julia RNG stream.  This restatement keeps the reference's draw ORDER inside
 * each logical unit (one NTC candidate, one convected particle, one merged
 * cell, ...), but gives every unit its own Philox stream so that results do
 * not depend on launch shape.  The device library uses the same stream layout;
 * it is described here once:
 *
 *   key     = (seed_lo32, seed_hi32)
 *   counter = (block, a, b, (tag << 28) | (sub << 24) | (step & 0xFFFFFF))
 *
 * Draw number n of a stream uses Philox block n >> 1 and the 64-bit word
 * (x[2e] | x[2e+1] << 32), e = n & 1.  A uniform double in [0, 1) is built
 * from the top 52 bits exactly like Julia's rand(Float64): [1, 2) - 1.
 */
#ifndef MERZ_ORACLE_PHILOX_REF_H
#define MERZ_ORACLE_PHILOX_REF_H

#include <stdint.h>
#include <string.h>

enum {
    ORC_TAG_NCOLL = 0,     /* a = cell rng id, b = 0, sub = pair code          */
    ORC_TAG_CAND = 1,      /* a = cell rng id, b = candidate #, sub = pair code */
    ORC_TAG_CONVECT = 2,   /* a = cell rng id, b = local index j, sub = species */
    ORC_TAG_MERGE = 3,     /* a = cell rng id, b = 0, sub = species             */
    ORC_TAG_SAMPLE = 4,    /* a = cell rng id, b = particle #, sub = species    */
    ORC_TAG_SAMPLE_CELL = 5 /* a = cell rng id, b = 0, sub = species           */
};

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
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

typedef struct {
    uint32_t key[2];
    uint32_t a, b, c3;
    uint64_t n;       /* next draw number */
    uint32_t buf[4];
    uint64_t buf_block; /* block held in buf, or UINT64_MAX */
} orc_stream;

static inline orc_stream orc_stream_make(uint64_t seed, uint32_t tag, uint32_t sub, uint64_t step,
                                         uint32_t a, uint32_t b)
{
    orc_stream s;
    s.key[0] = (uint32_t)seed;
    s.key[1] = (uint32_t)(seed >> 32);
    s.a = a;
    s.b = b;
    s.c3 = ((tag & 0xFu) << 28) | ((sub & 0xFu) << 24) | ((uint32_t)step & 0xFFFFFFu);
    s.n = 0;
    s.buf_block = UINT64_MAX;
    return s;
}

static inline uint64_t orc_stream_bits(orc_stream* s)
{
    uint64_t blk = s->n >> 1;
    unsigned e = (unsigned)(s->n & 1u);
    if (blk != s->buf_block) {
        uint32_t ctr[4] = {(uint32_t)blk, s->a, s->b, s->c3};
        orc_philox4x32_10(ctr, s->key, s->buf);
        s->buf_block = blk;
    }
    s->n++;
    return (uint64_t)s->buf[2 * e] | ((uint64_t)s->buf[2 * e + 1] << 32);
}

/* uniform in [0, 1), multiples of 2^-52 (Julia rand(Float64) construction) */
static inline double orc_stream_uniform(orc_stream* s)
{
    uint64_t bits = orc_stream_bits(s);
    uint64_t m = 0x3FF0000000000000ull | (bits >> 12);
    double d;
    memcpy(&d, &m, sizeof d);
    return d - 1.0;
}

#endif
