/*
 * philox.h -- ORACLE (test infrastructure, never linked into the product).
 *
 * Philox-4x32-10 counter-based generator, written from the published
 * description in Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11 (multiplier and Weyl constants as given there).  The
 * product's CUDA kernels carry their own implementation; both are checked
 * against the paper's known-answer vectors by the test suite.
 *
 * Stream layout shared with the kernels: key = 64-bit SEED, counter =
 * {block, step, particle index, stage}; each block yields four 32-bit words
 * consumed in order.
 */
#ifndef IMC_ORACLE_PHILOX_H_
#define IMC_ORACLE_PHILOX_H_
#include <stdint.h>
#include <math.h>

#define ORC_PHILOX_M0 0xD2511F53u
#define ORC_PHILOX_M1 0xCD9E8D57u
#define ORC_PHILOX_W0 0x9E3779B9u
#define ORC_PHILOX_W1 0xBB67AE85u

enum { ORC_STAGE_TRANSPORT = 0, ORC_STAGE_SOURCE = 1, ORC_STAGE_SURR_DATA = 3, ORC_STAGE_SURR_TEST = 4 };

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)ORC_PHILOX_M0 * (uint64_t)c0;
        uint64_t p1 = (uint64_t)ORC_PHILOX_M1 * (uint64_t)c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += ORC_PHILOX_W0; k1 += ORC_PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* One particle's stream for one stage of one step. */
typedef struct OrcStream {
    uint32_t key[2];
    uint32_t ctr[4];
    uint32_t buf[4];
    int idx;
} OrcStream;

static inline void orc_stream_init(OrcStream *s, uint64_t seed, uint32_t step, uint32_t pid, uint32_t stage) {
    s->key[0] = (uint32_t)seed; s->key[1] = (uint32_t)(seed >> 32);
    s->ctr[0] = 0; s->ctr[1] = step; s->ctr[2] = pid; s->ctr[3] = stage;
    s->idx = 4;
}

static inline uint32_t orc_next_u32(OrcStream *s) {
    if (s->idx == 4) {
        orc_philox4x32_10(s->ctr, s->key, s->buf);
        s->ctr[0] += 1u;
        s->idx = 0;
    }
    return s->buf[s->idx++];
}

/* uniform on [0,1): 24-bit grid (float) / 53-bit grid (double, high word first) */
static inline float orc_rand_f32(OrcStream *s) {
    return (float)(orc_next_u32(s) >> 8) * 0x1p-24f;
}
static inline double orc_rand_f64(OrcStream *s) {
    uint64_t hi = orc_next_u32(s);
    uint64_t lo = orc_next_u32(s);
    return (double)(((hi << 32) | lo) >> 11) * 0x1p-53;
}
/* exponential variate -log(v) (the reference's randexp), v an odd multiple of
 * 2^-24 (2^-53) on (0,1), so the variate is never 0 and never infinite */
static inline float orc_randexp_f32(OrcStream *s) {
    float v = (float)((orc_next_u32(s) >> 8) | 1u) * 0x1p-24f;
    return -logf(v);
}
static inline double orc_randexp_f64(OrcStream *s) {
    uint64_t hi = orc_next_u32(s);
    uint64_t lo = orc_next_u32(s);
    double v = (double)((((hi << 32) | lo) >> 11) | 1u) * 0x1p-53;
    return -log(v);
}

#endif
