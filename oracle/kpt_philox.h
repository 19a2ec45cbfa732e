/*
 * Counter-based Philox4x32-10 noise stream used by the oracle (test
 * infrastructure only; the product carries its own CUDA implementation).
 *
 * Algorithm: Philox4x32 with 10 rounds, Salmon, Moraes, Dror, Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3", SC'11.  Multipliers
 * 0xD2511F53 / 0xCD9E8D57, Weyl key increments 0x9E3779B9 / 0xBB67AE85.
 *
 * Stream layout (identical on the GPU side):
 *   key     = (seed & 0xffffffff, seed >> 32)
 *   counter = (block, index, frame, tag)
 *   draw n of a stream uses block n/2, words 2*(n%2) (low) and
 *   2*(n%2)+1 (high); u = ((high << 32 | low) >> 11) * 2^-53 in [0, 1).
 * The reference draws XorShift64 states per thread
 * (RandomManager.hpp:13-62); its order depends on scheduling, so this
 * keyed stream replaces it on both sides of every parity comparison.
 */
#ifndef KPT_ORACLE_PHILOX_H
#define KPT_ORACLE_PHILOX_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    KPT_ORACLE_TAG_INJECT = 1u,
    KPT_ORACLE_TAG_PUSH = 2u,
    KPT_ORACLE_TAG_LIBRARY = 3u,
    KPT_ORACLE_TAG_GENERATOR = 4u,
    KPT_ORACLE_TAG_OTHER = 255u
};

static inline void kpt_oracle_philox4x32_10(const uint32_t counter[4],
                                            const uint32_t key[2],
                                            uint32_t out[4]) {
    uint32_t c0 = counter[0], c1 = counter[1], c2 = counter[2], c3 = counter[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* One keyed stream: (seed, index, frame, tag) plus a running draw count. */
typedef struct {
    uint32_t key[2];
    uint32_t index;
    uint32_t frame;
    uint32_t tag;
    uint64_t draw;
    uint32_t block[4];
} kpt_oracle_stream;

static inline void kpt_oracle_stream_init(kpt_oracle_stream* s, uint64_t seed,
                                          uint32_t index, uint32_t frame,
                                          uint32_t tag) {
    s->key[0] = (uint32_t)seed;
    s->key[1] = (uint32_t)(seed >> 32);
    s->index = index;
    s->frame = frame;
    s->tag = tag;
    s->draw = 0;
}

/* Next uniform double in [0, 1). */
static inline double kpt_oracle_stream_u01(kpt_oracle_stream* s) {
    const uint64_t n = s->draw++;
    if ((n & 1u) == 0u) {
        const uint32_t counter[4] = {(uint32_t)(n >> 1), s->index, s->frame, s->tag};
        kpt_oracle_philox4x32_10(counter, s->key, s->block);
    }
    const uint32_t lo = s->block[(n & 1u) * 2u];
    const uint32_t hi = s->block[(n & 1u) * 2u + 1u];
    const uint64_t bits = (((uint64_t)hi << 32) | (uint64_t)lo) >> 11;
    return (double)bits * (1.0 / 9007199254740992.0);
}

#ifdef __cplusplus
}
#endif

#endif
