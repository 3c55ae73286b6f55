/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Nothing in the product library includes
 * this file; only the CPU oracle (oracle/ug_oracle.cpp) and the reference
 * harness (oracle/ref_harness/) do.
 *
 * Counter-based noise streams shared by the oracle and the reference harness.
 *
 * The reference draws every random number from one std::mt19937 per MPI rank
 * (c++/src/poisson_noise.cpp:3-38, seeded 15000+1000*rank at
 * c++/src/NetworkGrowthSimulator.cpp:2435-2446), so its trajectories depend on
 * the rank count and on the order in which neurons are stepped.  The rebuild
 * replaces that generator by independent Philox4x32-10 streams (Salmon,
 * Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11),
 * one per (network, trial, neuron, purpose), so that any execution order gives
 * the same draws.  The conversions from a 32-bit word to the reference's
 * random quantities keep the reference's formulas:
 *   get_spike_time(lambda) = -log(1 - u/0xffffffff) / lambda   (poisson_noise.cpp:14-20)
 *   random(G)              = (G * u) / 0xffffffff                (poisson_noise.cpp:22-25)
 *   point-distribution index in [0,30): (u * 30) >> 32           (replaces
 *                            uniform_int_distribution(0,29), poisson_noise.cpp:27-30)
 *
 * Stream layout (the CUDA kernels use the same layout, written separately):
 *   key     = (seed & 0xffffffff, seed >> 32)
 *   counter = (block, entity, trial, (kind << 24) | net)
 *   word n of a stream = philox(counter with block = n / 4)[n % 4]
 */
#ifndef UGO_NOISE_H
#define UGO_NOISE_H

#include <stdint.h>

enum {
    UGO_KIND_RA_WHITE = 1,    /* HVC(RA) white-noise point distribution, 4 words per step */
    UGO_KIND_I_POISSON = 2,   /* HVC(I) Poisson conductance noise, sequential words */
    UGO_KIND_TRIAL = 3,       /* per-trial network draws (mean injection time) */
    UGO_KIND_REPLACE = 4,     /* neuron replacement resampling */
    UGO_KIND_TOPOLOGY = 6     /* network topology generation (coordinates, RA<->I connections) */
};

static inline uint32_t ugo_mulhilo32(uint32_t a, uint32_t b, uint32_t* hi)
{
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    return (uint32_t)p;
}

/* Philox4x32 with 10 rounds (Salmon et al. 2011, section 3.2). */
static inline void ugo_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; ++round) {
        uint32_t hi0, hi1;
        uint32_t lo0 = ugo_mulhilo32(0xD2511F53u, c0, &hi0);
        uint32_t lo1 = ugo_mulhilo32(0xCD9E8D57u, c2, &hi1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct {
    uint32_t key[2];
    uint32_t ctr[4];   /* ctr[0] is replaced by the block index on each refill */
    uint32_t buf[4];
    uint64_t next;     /* index of the next word */
} ugo_stream;

static inline void ugo_stream_init(ugo_stream* s, uint64_t seed, uint32_t kind, uint32_t net,
                                   uint32_t entity, uint32_t trial)
{
    s->key[0] = (uint32_t)(seed & 0xffffffffu);
    s->key[1] = (uint32_t)(seed >> 32);
    s->ctr[0] = 0;
    s->ctr[1] = entity;
    s->ctr[2] = trial;
    s->ctr[3] = (kind << 24) | (net & 0xffffffu);
    s->next = 0;
}

static inline uint32_t ugo_stream_word(ugo_stream* s)
{
    uint32_t lane = (uint32_t)(s->next & 3u);
    if (lane == 0) {
        uint32_t c[4] = { (uint32_t)(s->next >> 2), s->ctr[1], s->ctr[2], s->ctr[3] };
        ugo_philox4x32_10(c, s->key, s->buf);
    }
    s->next++;
    return s->buf[lane];
}

static inline double ugo_u01(uint32_t u) { return (double)u / 4294967295.0; }
static inline double ugo_random_G(double G, uint32_t u) { return (G * (double)u) / 4294967295.0; }
static inline int ugo_point_index(uint32_t u) { return (int)(((uint64_t)u * 30u) >> 32); }

#endif
