// Counter-based noise streams (Philox4x32-10, Salmon et al., SC'11) used by
// the kernels and by the host (per-trial draws, replacement resampling).
//
// They replace the reference's single per-rank std::mt19937
// (c++/src/poisson_noise.cpp:3-38) so that every neuron's noise is a function
// of (seed, network, trial, neuron, word index) and not of the order in which
// neurons are stepped.  Layout:
//   key     = (seed low 32 bits, seed high 32 bits)
//   counter = (word / 4, entity, trial, (kind << 24) | network)
//   word n  = philox(counter)[n % 4]
// Conversions keep the reference's formulas (poisson_noise.cpp:14-30):
//   get_spike_time(lambda) = -log(1 - u / 0xffffffff) / lambda
//   random(G)              = G * u / 0xffffffff
//   point index in [0,30)  = (u * 30) >> 32
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define UG_HD __host__ __device__ __forceinline__
#else
#define UG_HD inline
#endif

namespace ug {

enum NoiseKind : uint32_t {
    kNoiseRAWhite = 1,    // HVC(RA) white noise: 4 words per integration step
    kNoiseIPoisson = 2,   // HVC(I) Poisson conductance noise: sequential words
    kNoiseTrial = 3,      // per-trial network draws (mean training injection time)
    kNoiseReplace = 4,    // neuron replacement resampling
    kNoiseCreate = 5,     // network set-up draws (the growth CLI's weight resampling)
    kNoiseTopology = 6    // topology generation: coordinates and RA<->I connections
};

struct Philox4 { uint32_t x, y, z, w; };

UG_HD Philox4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#if defined(__CUDA_ARCH__)
        const uint32_t hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
#else
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
        const uint32_t n0 = hi1 ^ c1 ^ k0;
        const uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return Philox4{c0, c1, c2, c3};
}

struct StreamId {
    uint32_t k0, k1, entity, trial, tag;
};

UG_HD StreamId make_stream(uint64_t seed, uint32_t kind, uint32_t net, uint32_t entity, uint32_t trial)
{
    return StreamId{(uint32_t)(seed & 0xffffffffu), (uint32_t)(seed >> 32), entity, trial, (kind << 24) | (net & 0xffffffu)};
}

UG_HD Philox4 stream_block(const StreamId& s, uint32_t block)
{
    return philox4x32_10(block, s.entity, s.trial, s.tag, s.k0, s.k1);
}

UG_HD uint32_t stream_word(const StreamId& s, uint32_t n)
{
    const Philox4 b = stream_block(s, n >> 2);
    const uint32_t lane = n & 3u;
    return lane == 0 ? b.x : lane == 1 ? b.y : lane == 2 ? b.z : b.w;
}

UG_HD double u01(uint32_t u) { return (double)u / 4294967295.0; }
UG_HD double random_G(double G, uint32_t u) { return (G * (double)u) / 4294967295.0; }
UG_HD int point_index(uint32_t u) { return (int)(((uint64_t)u * 30u) >> 32); }

// Host-side sequential reader of one stream (per-trial draws, replacement).
struct HostStream {
    StreamId id;
    uint32_t next;
    uint32_t word() { return stream_word(id, next++); }
};

}  // namespace ug
