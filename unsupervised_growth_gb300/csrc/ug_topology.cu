// Network topology generation on the device: createNetworkForGrowth, i.e.
// NetworkGrowthSimulator::generate_network_topology (c++/src/NetworkGrowthSimulator.cpp:110-155)
// with sample_coordinates (:222-403), sample_connections (:620-705), p_RA2I / p_I2RA
// (:707-719) and write_different_training_arrangements (:406-457).
//
// The reference makes every draw from its rank's mt19937 in program order.  Here each
// draw has its own place in the topology streams (kind kNoiseTopology; the trial field
// names the purpose), so the sequential loops become parallel ones with the same result:
//
// * Interneurons.  Interneuron i's r-th try uses words 2r, 2r+1 of stream i.  Every first
//   try is checked against all earlier ones at once (a warp per interneuron over the grid);
//   from the first that is too close on, one block lets it draw again until it fits and
//   then searches the next conflict among the later ones, until there is none.
// * HVC(RA) placement.  The a-th attempt uses stream entity a, so the reference's loop
//   (attempt until far enough from every interneuron and every earlier HVC(RA)) keeps
//   exactly the attempts that are far enough from every interneuron and every attempt
//   kept before them.  Batches of K attempts: each attempt against all points kept so far
//   (k_ra_check_fixed), each pair inside the batch (k_ra_check_batch, which records the
//   conflicts), then one block decides the batch in attempt order (k_ra_resolve).  The
//   result does not depend on K; K is sized so that an attempt has about one conflict
//   inside its batch, and a batch with more than kMaxPartners is run again with a smaller K.
// * Connections.  One warp per source row; a lane decides four targets from one Philox
//   block (word j of row i's stream decides the pair (i, j)).  Two passes (decide into
//   4-bit masks and row counts; scan; fill) give the reference's order, by source then
//   target.  A pair whose draw is at least the amplitude A is rejected without evaluating
//   the Gaussian (A * exp(-d^2 / 2 sigma^2) never exceeds A).
// * Training arrangements (n_tr neurons) are chosen on the host from the coordinates.
//
// This unit is compiled without multiply-add contraction, so its dot products round
// exactly as the host's do; acos, exp, sin and cos are CUDA's.
#include "ug_philox.cuh"
#include "ug_topology.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kExpDist = 40.0;   // EXPERIMENTAL_INTERNEURON_DISTANCE (NetworkGrowthSimulator.cpp:19)
constexpr double kMinDist = 10.0;   // MIN_INTERSOMATIC_DISTANCE (:20)
constexpr double kShift = 0.15;     // interneuron jitter in model spacings (sample_coordinates :224)
constexpr int kMaxPartners = 16;    // conflicts one attempt may have inside its batch
constexpr int kMaxBatch = 16384;
constexpr int kMinBatch = 64;
constexpr int kResolveThreads = 1024;
constexpr int kChunk = 256;         // points staged in shared memory per block
constexpr int kCheckThreads = 128;
constexpr int kRowThreads = 256;    // 8 rows per block in the connection kernels
constexpr int kMaxRetry = 1 << 16;  // re-tries of one interneuron before giving up
constexpr long long kMaxMisses = 1 << 16;   // attempts rejected in a row before the placement gives up
// the trial field of the topology streams
constexpr uint32_t kPartInterneuron = 0, kPartPlacement = 1, kPartRA2I = 2, kPartI2RA = 3, kPartTraining = 4;

struct Geo {
    int sphere;
    int side;             // square: floor(sqrt(N_I)) interneurons per grid row
    double model;         // MODEL_INTERNEURON_DISTANCE
    double too_close;     // model * MIN_INTERSOMATIC_DISTANCE / EXPERIMENTAL_INTERNEURON_DISTANCE
    double lo, hi;        // prefilter bounds: dot products (sphere) or squared distances (square)
    float lo32, hi32;     // the same bounds for single-precision copies of the coordinates
    double root;          // sqrt(N_I)
    uint64_t seed;
    uint32_t net;
};

// device-side progress of the placement, read back after each batch
struct State {
    int count;            // HVC(RA) placed
    int overflow;         // a batch attempt had more than kMaxPartners conflicts
    int status;           // 1: an interneuron found no place
    int first;            // the first interneuron whose first try is too close to an earlier one
    int kept;             // attempts kept by the last batch (before the cut at N_RA)
    int unflagged;        // attempts of the last batch far enough from the points placed before it
    long long attempts;   // attempts consumed
    long long last_kept;  // attempts consumed up to the last kept one
    long long retries;    // interneuron re-tries
};

__host__ __device__ inline double dot3(const double* a, const double* b)
{
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// distance_on_sphere (NetworkGrowthSimulator.cpp:36-44) or distance2d (:31-34)
__host__ __device__ inline double dist(const Geo& g, const double* a, const double* b)
{
    if (g.sphere) {
        const double t = dot3(a, b);
        return t > 1.0 ? 0.0 : acos(t);
    }
    return sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]));
}

// dist(a, b) < too_close; pairs far from the bound are decided by the dot product or the
// squared distance alone (the bounds sit 1e-9 off it, far outside acos' rounding)
__device__ inline bool too_close(const Geo& g, const double* a, const double* b)
{
    if (g.sphere) {
        const double t = dot3(a, b);
        if (t < g.lo) return false;
        if (t > g.hi) return true;
    } else {
        const double d2 = (a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]);
        if (d2 > g.hi) return false;
        if (d2 < g.lo) return true;
    }
    return dist(g, a, b) < g.too_close;
}

// The single-precision prefilter: 0 far, 1 too close, 2 undecided.  The copies differ
// from the doubles by at most 2^-24 relative, so a dot product of unit vectors is off by
// less than 3e-7 and a distance on the unit square by less than 5e-7; the bounds sit
// 2e-6 (sphere) and 1e-6 (square) off the threshold.
__device__ inline int close32(const Geo& g, float4 a, float4 b)
{
    if (g.sphere) {
        const float t = __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
        return t < g.lo32 ? 0 : t > g.hi32 ? 1 : 2;
    }
    const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y);
    const float d2 = __fmaf_rn(dy, dy, __fmul_rn(dx, dx));
    return d2 > g.hi32 ? 0 : d2 < g.lo32 ? 1 : 2;
}

__device__ inline float4 to32(const double* p) { return make_float4((float)p[0], (float)p[1], (float)p[2], 0.f); }

// too_close(a, b) decided on the copies where they suffice
__device__ inline bool close_mixed(const Geo& g, float4 a32, float4 b32, const double* a, const double* b)
{
    const int c = close32(g, a32, b32);
    return c == 2 ? too_close(g, a, b) : c == 1;
}

// inclusive scan over a block of blockDim.x (a multiple of 32, at most 1024) threads
__device__ inline int block_scan(int v, int* total, int* wsum)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int s = lane < nw ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) wsum[lane] = s;
    }
    __syncthreads();
    const int out = x + (warp > 0 ? wsum[warp - 1] : 0);
    *total = wsum[nw - 1];
    __syncthreads();
    return out;
}

// interneuron i's r-th try on the sphere (:314-338)
__device__ void i_try(const Geo& g, int i, uint32_t r, double z, double phi, double* t)
{
    const ug::Philox4 b =
        ug::stream_block(ug::make_stream(g.seed, ug::kNoiseTopology, g.net, (uint32_t)i, kPartInterneuron), r >> 1);
    const uint32_t u0 = (r & 1) ? b.z : b.x, u1 = (r & 1) ? b.w : b.y;
    const double theta = acos(z);
    const double theta_noise = -kShift * g.model + ug::random_G(2 * kShift * g.model, u0);
    const double phi_noise = (-kShift * g.model + ug::random_G(2 * kShift * g.model, u1)) / sin(theta);
    t[0] = cos(phi + phi_noise) * sin(theta + theta_noise);
    t[1] = sin(phi + phi_noise) * sin(theta + theta_noise);
    t[2] = cos(theta + theta_noise);
}

// every interneuron's first try on the sphere, at its point of the Fibonacci lattice
// (base: z and phi as :296-300 accumulate them); the square grid (:231-241), whose side^2
// jittered points are final and whose remaining interneurons stay at the origin
__global__ void k_i_first_tries(Geo g, int n_i, const double* base, double* xyz, float4* xyz32, State* st)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q == 0) st->first = n_i;
    if (q >= n_i) return;
    if (g.sphere) {
        i_try(g, q, 0, base[2 * q], base[2 * q + 1], xyz + 3 * q);
    } else if (q < g.side * g.side) {
        const int i = q / g.side, k = q % g.side;
        const ug::Philox4 b =
            ug::stream_block(ug::make_stream(g.seed, ug::kNoiseTopology, g.net, (uint32_t)q, kPartInterneuron), 0);
        xyz[3 * q] = (double)(i + 1) / (g.root + 1) - kShift * g.model + ug::random_G(2 * kShift * g.model, b.x);
        xyz[3 * q + 1] = (double)(k + 1) / (g.root + 1) - kShift * g.model + ug::random_G(2 * kShift * g.model, b.y);
        xyz[3 * q + 2] = 0.0;
    } else {
        xyz[3 * q] = xyz[3 * q + 1] = xyz[3 * q + 2] = 0.0;
    }
    xyz32[q] = to32(xyz + 3 * q);
}

// st->first = the first interneuron whose first try is too close to an earlier one's;
// a warp per interneuron, the longest rows first
__global__ void __launch_bounds__(kRowThreads) k_i_scan(Geo g, int n_i, const double* xyz, const float4* xyz32,
                                                        State* st)
{
    const int lane = threadIdx.x & 31;
    const int i = n_i - 1 - (blockIdx.x * (kRowThreads / 32) + (threadIdx.x >> 5));
    if (i < 1) return;
    const int first = __shfl_sync(0xffffffffu, *(volatile int*)&st->first, 0);
    if (i >= first) return;
    const float4 a = xyz32[i];
    bool c = false;
    for (int j = lane; j < i && !c; j += 32) c = close_mixed(g, a, xyz32[j], xyz + 3 * i, xyz + 3 * j);
    if (__any_sync(0xffffffffu, c) && lane == 0) atomicMin(&st->first, i);
}

// the sequential part of the interneuron placement (sphere), from the first conflict on:
// the conflicting interneuron draws again until it fits, then the next conflict among
// the later ones is searched, until there is none (one block)
__global__ void __launch_bounds__(1024) k_interneurons(Geo g, int n_i, double* xyz, float4* xyz32, const double* base,
                                                       State* st)
{
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nth >> 5;
    __shared__ int s_first, s_close;
    long long retries = 0;
    int f = st->first;
    while (f < n_i) {
        // every try before it stands; it draws again until it fits
        bool placed = false;
        for (int r = 1; r <= kMaxRetry; ++r) {
            double t[3];
            i_try(g, f, (uint32_t)r, base[2 * f], base[2 * f + 1], t);
            const float4 t32 = to32(t);
            if (tid == 0) s_close = 0;
            __syncthreads();
            for (int j = tid; j < f; j += nth)
                if (close_mixed(g, t32, xyz32[j], t, xyz + 3 * j)) s_close = 1;
            __syncthreads();
            const int cl = s_close;
            __syncthreads();
            ++retries;
            if (!cl) {
                if (tid == 0) {
                    xyz[3 * f] = t[0];
                    xyz[3 * f + 1] = t[1];
                    xyz[3 * f + 2] = t[2];
                    xyz32[f] = t32;
                }
                placed = true;
                break;
            }
        }
        if (!placed) {
            if (tid == 0) st->status = 1;
            return;
        }
        __syncthreads();
        // the first later interneuron whose try is too close to an earlier one
        if (tid == 0) s_first = n_i;
        __syncthreads();
        for (int i = f + 1 + warp; i < n_i; i += nwarps) {
            const int first = __shfl_sync(0xffffffffu, *(volatile int*)&s_first, 0);
            if (i >= first) break;
            const float4 a = xyz32[i];
            bool c = false;
            for (int j = lane; j < i && !c; j += 32) c = close_mixed(g, a, xyz32[j], xyz + 3 * i, xyz + 3 * j);
            if (__any_sync(0xffffffffu, c)) {
                if (lane == 0) atomicMin(&s_first, i);
                break;
            }
        }
        __syncthreads();
        f = s_first;
        __syncthreads();
    }
    if (tid == 0) st->retries = retries;
}

// HVC(RA) attempts a0 .. a0+K-1 (:342-350; the square's :247-248)
__global__ void k_ra_candidates(Geo g, uint32_t a0, int K, double* cand, float4* cand32, int* flag, int* npart)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const ug::Philox4 b = ug::stream_block(
        ug::make_stream(g.seed, ug::kNoiseTopology, g.net, a0 + (uint32_t)k, kPartPlacement), 0);
    if (g.sphere) {
        const double zz = 2 * ug::random_G(1.0, b.x) - 1;
        const double ph = ug::random_G(2.0 * kPi, b.y);
        cand[3 * k] = sin(acos(zz)) * cos(ph);
        cand[3 * k + 1] = sin(acos(zz)) * sin(ph);
        cand[3 * k + 2] = zz;
    } else {
        cand[3 * k] = 0.5 / (g.root + 1) + ug::random_G(1.0 - 1.0 / (g.root + 1), b.x);
        cand[3 * k + 1] = 0.5 / (g.root + 1) + ug::random_G(1.0 - 1.0 / (g.root + 1), b.y);
        cand[3 * k + 2] = 0.0;
    }
    cand32[k] = to32(cand + 3 * k);
    flag[k] = 0;
    npart[k] = 0;
}

// flag[k] = attempt k is too close to an interneuron or to an HVC(RA) placed before the batch;
// blockIdx.y picks a chunk of those points
__global__ void __launch_bounds__(kCheckThreads) k_ra_check_fixed(Geo g, const double* cand, const float4* cand32,
                                                                  int K, const double* i_xyz, const float4* i32,
                                                                  int n_i, const double* ra_xyz, const float4* ra32,
                                                                  int count, int* flag)
{
    __shared__ float4 sp[kChunk];
    const int c0 = blockIdx.y * kChunk, cn = min(kChunk, n_i + count - c0);
    for (int q = threadIdx.x; q < cn; q += blockDim.x) {
        const int p = c0 + q;
        sp[q] = p < n_i ? i32[p] : ra32[p - n_i];
    }
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K || *(volatile int*)(flag + k)) return;
    const float4 a = cand32[k];
    for (int q = 0; q < cn; ++q) {
        const int c = close32(g, a, sp[q]);
        if (c == 0) continue;
        const int p = c0 + q;
        if (c == 1 || too_close(g, cand + 3 * k, p < n_i ? i_xyz + 3 * p : ra_xyz + 3 * (p - n_i))) {
            flag[k] = 1;
            return;
        }
    }
}

// conflicts between unflagged attempts j < k of the batch; blockIdx.y picks the chunk of j
__global__ void __launch_bounds__(kCheckThreads) k_ra_check_batch(Geo g, const double* cand, const float4* cand32,
                                                                  int K, const int* flag, int* part, int* npart,
                                                                  State* st)
{
    __shared__ float4 sp[kChunk];
    __shared__ int sf[kChunk];
    const int j0 = blockIdx.y * kChunk, kb = blockIdx.x * blockDim.x;
    if (j0 >= kb + (int)blockDim.x - 1) return;   // no j below any k of this block
    const int jn = min(kChunk, K - j0);
    for (int q = threadIdx.x; q < jn; q += blockDim.x) {
        sp[q] = cand32[j0 + q];
        sf[q] = flag[j0 + q];
    }
    __syncthreads();
    const int k = kb + threadIdx.x;
    if (k >= K || flag[k]) return;
    const float4 a = cand32[k];
    const int jend = min(jn, k - j0);
    for (int q = 0; q < jend; ++q) {
        if (sf[q] || !close_mixed(g, a, sp[q], cand + 3 * k, cand + 3 * (j0 + q))) continue;
        const int slot = atomicAdd(npart + k, 1);
        if (slot < kMaxPartners)
            part[k * kMaxPartners + slot] = j0 + q;
        else
            st->overflow = 1;
    }
}

// keeps, in attempt order, every unflagged attempt none of whose earlier conflicts was
// kept, and appends the first (N_RA - count) of them to the placed HVC(RA)
__global__ void __launch_bounds__(kResolveThreads) k_ra_resolve(const double* cand, const float4* cand32, int K,
                                                                const int* flag, const int* part, const int* npart,
                                                                int n_ra, uint32_t a0, double* ra_xyz, float4* ra32,
                                                                State* st)
{
    __shared__ unsigned char s_state[kMaxBatch];   // 0 open, 1 kept, 2 rejected
    __shared__ int wsum[32];
    volatile unsigned char* vs = s_state;
    if (st->overflow) return;
    const int tid = threadIdx.x;
    const int count = st->count;
    const int per = (K + kResolveThreads - 1) / kResolveThreads;
    const int k0 = tid * per;   // contiguous attempts per thread, for the ordered scan
    for (int m = 0; m < per; ++m)
        if (k0 + m < K) s_state[k0 + m] = flag[k0 + m] ? 2 : 0;
    __syncthreads();
    for (int round = 0; round < K; ++round) {
        int open = 0;
        for (int m = 0; m < per; ++m) {
            const int k = k0 + m;
            if (k >= K || vs[k] != 0) continue;
            const int np = npart[k];
            bool blocked = false, ready = true;
            for (int p = 0; p < np && !blocked; ++p) {
                const unsigned char s = vs[part[k * kMaxPartners + p]];
                blocked = s == 1;
                ready = ready && s != 0;
            }
            if (blocked)
                vs[k] = 2;
            else if (ready)
                vs[k] = 1;
            else
                open = 1;
        }
        if (!__syncthreads_or(open)) break;
    }
    int mine = 0, open = 0;
    for (int m = 0; m < per; ++m) {
        if (k0 + m >= K) continue;
        mine += s_state[k0 + m] == 1;
        open += flag[k0 + m] == 0;
    }
    int total = 0, unflagged = 0;
    int rank = block_scan(mine, &total, wsum) - mine;
    block_scan(open, &unflagged, wsum);
    const int remaining = n_ra - count, placed = min(total, remaining);
    for (int m = 0; m < per; ++m) {
        const int k = k0 + m;
        if (k >= K || s_state[k] != 1) continue;
        if (rank < remaining) {
            ra_xyz[3 * (count + rank)] = cand[3 * k];
            ra_xyz[3 * (count + rank) + 1] = cand[3 * k + 1];
            ra_xyz[3 * (count + rank) + 2] = cand[3 * k + 2];
            ra32[count + rank] = cand32[k];
            if (rank == placed - 1) st->last_kept = (long long)a0 + k + 1;
        }
        ++rank;
    }
    __syncthreads();
    if (tid == 0) {
        st->count = count + placed;
        st->kept = total;
        st->unflagged = unflagged;
        st->attempts = total >= remaining ? st->last_kept : (long long)a0 + K;
    }
}

// One direction's connection probability A exp(-d^2 / (2 sigma^2)) (p_RA2I / p_I2RA, :707-719)
// with what the single-precision prefilter needs.
struct Gauss {
    double A, sigma_square;
    long long wA;   // random(1) < A exactly when the pair's word is below wA
    float logA;     // log(A)
    float scale;    // EXPERIMENTAL_INTERNEURON_DISTANCE / model
    float inv2s2;   // 1 / (2 sigma^2)
    float rel;      // relative half-width of the band decided in double precision
    int exact;      // 1: every pair below wA in double precision
};

// the reference's test (:651-652): random(1) < A exp(-d^2 / (2 sigma^2)), in double precision
__device__ inline bool connect_exact(const Geo& g, const Gauss& q, const double* a, const double* b, uint32_t w)
{
    const double d = dist(g, a, b) * kExpDist / g.model;
    return ug::random_G(1, w) < q.A * exp(-d * d / (2 * q.sigma_square));
}

// The same test on the single-precision copies where a margin decides it.  With
// x = d^2 / (2 sigma^2) and L = log(A / random(1)) a pair connects when x < L.  Every
// HVC(RA)-interneuron pair is at least the minimum distance t apart, so the copies give
// d to a relative 4e-7 / (t sin t) on the sphere (1e-6 / t on the square), x to twice that,
// and L to 1e-5; pairs with |x - L| inside rel * max(|x|, |L|) + 1e-3 (rel >= 0.02 plus
// those bounds) and the word 0 (random(1) = 0) are decided in double precision.
__device__ inline bool connect(const Geo& g, const Gauss& q, float4 a32, float4 b32, const double* a, const double* b,
                               uint32_t w)
{
    if (q.exact || w == 0) return connect_exact(g, q, a, b, w);
    float d;
    if (g.sphere) {
        const float t = __fmaf_rn(a32.z, b32.z, __fmaf_rn(a32.y, b32.y, __fmul_rn(a32.x, b32.x)));
        d = __fmul_rn(acosf(fminf(fmaxf(t, -1.f), 1.f)), q.scale);
    } else {
        const float dx = __fsub_rn(a32.x, b32.x), dy = __fsub_rn(a32.y, b32.y);
        d = __fmul_rn(sqrtf(__fmaf_rn(dy, dy, __fmul_rn(dx, dx))), q.scale);
    }
    const float x = __fmul_rn(__fmul_rn(d, d), q.inv2s2);
    const float L = __fsub_rn(q.logA, logf(__fmul_rn((float)w, 2.3283064e-10f)));
    const float tol = __fmaf_rn(q.rel, fmaxf(fabsf(x), fabsf(L)), 1e-3f);
    if (x - L > tol) return false;
    if (L - x > tol) return true;
    return connect_exact(g, q, a, b, w);
}

// RA->I or I->RA decisions (:649-690) as bit words of 32 targets, and the per-row counts.
// A lane decides four targets from one Philox block, 128 targets per warp pass.
__global__ void __launch_bounds__(kRowThreads) k_conn_decide(Geo g, Gauss q, const double* src, const float4* src32,
                                                             int n_src, const double* dst, const float4* dst32,
                                                             int n_dst, uint32_t part, unsigned* bits, int nw,
                                                             int* rowcnt)
{
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (kRowThreads / 32) + (threadIdx.x >> 5);
    if (row >= n_src) return;
    const double* a = src + 3 * row;
    const float4 a32 = src32[row];
    const ug::StreamId s = ug::make_stream(g.seed, ug::kNoiseTopology, g.net, (uint32_t)row, part);
    int cnt = 0;
    for (int c0 = 0; c0 < n_dst; c0 += 128) {
        const int j0 = c0 + 4 * lane;
        unsigned m = 0;
        if (j0 < n_dst) {
            const ug::Philox4 b = ug::stream_block(s, (uint32_t)(j0 >> 2));
            const uint32_t w[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int j = j0 + c;
                if (j < n_dst && (long long)w[c] < q.wA && connect(g, q, a32, dst32[j], a, dst + 3 * j, w[c]))
                    m |= 1u << c;
            }
        }
        // lanes 8k .. 8k+7 make word k of this pass
        unsigned v = m << (4 * (lane & 7));
        v |= __shfl_xor_sync(0xffffffffu, v, 1);
        v |= __shfl_xor_sync(0xffffffffu, v, 2);
        v |= __shfl_xor_sync(0xffffffffu, v, 4);
        const int wi = (c0 >> 5) + (lane >> 3);
        if ((lane & 7) == 0 && wi < nw) bits[(size_t)row * nw + wi] = v;
        cnt += __popc(m);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0) rowcnt[row] = cnt;
}

// off[0..n] = exclusive prefix sums of cnt[0..n-1]
__global__ void __launch_bounds__(1024) k_scan(const int* cnt, int n, int* off)
{
    __shared__ int wsum[32];
    int carry = 0;
    for (int b = 0; b < n; b += blockDim.x) {
        const int i = b + threadIdx.x;
        const int v = i < n ? cnt[i] : 0;
        int total = 0;
        const int incl = block_scan(v, &total, wsum);
        if (i < n) off[i] = carry + incl - v;
        carry += total;
    }
    if (threadIdx.x == 0) off[n] = carry;
}

// targets and lengths of the kept pairs, by source then target
__global__ void __launch_bounds__(kRowThreads) k_conn_fill(Geo g, const double* src, int n_src, const double* dst,
                                                           const unsigned* bits, int nw, const int* off, int* tgt,
                                                           double* len)
{
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (kRowThreads / 32) + (threadIdx.x >> 5);
    if (row >= n_src) return;
    const double* a = src + 3 * row;
    int base = off[row];
    for (int w0 = 0; w0 < nw; w0 += 32) {
        const int wi = w0 + lane;
        unsigned m = wi < nw ? bits[(size_t)row * nw + wi] : 0u;
        const int c = __popc(m);
        int incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        int pos = base + incl - c;
        while (m) {
            const int j = 32 * wi + __ffs(m) - 1;
            m &= m - 1;
            tgt[pos] = j;
            len[pos] = dist(g, a, dst + 3 * j) * kExpDist / g.model;
            ++pos;
        }
        base += __shfl_sync(0xffffffffu, incl, 31);
    }
}

// ------------------------------------------------------------------ host side

ug_status terr(ug_status s, const std::string& msg)
{
    ug_set_last_error(msg);
    return s;
}

#define TCUDA(call)                                                                                \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return terr(e_ == cudaErrorMemoryAllocation ? UG_ENOMEM : UG_ECUDA,                    \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                       \
    } while (0)

// stream-ordered device scratch, returned to the pool when the generation ends
class Scratch {
public:
    explicit Scratch(cudaStream_t st) : st_(st) {}
    ~Scratch()
    {
        for (void* p : ptrs_) cudaFreeAsync(p, st_);
    }
    template <class T>
    cudaError_t get(T** p, size_t n)
    {
        void* q = nullptr;
        const cudaError_t e = cudaMallocAsync(&q, std::max<size_t>(n, 1) * sizeof(T), st_);
        if (e == cudaSuccess) ptrs_.push_back(q);
        *p = (T*)q;
        return e;
    }

private:
    cudaStream_t st_;
    std::vector<void*> ptrs_;
};

double model_distance(int arrangement, int n_i)
{
    if (arrangement == UG_ARRANGEMENT_SQUARE) return 1 / (std::sqrt((double)n_i) + 1);
    // the first two points of the Fibonacci lattice (:296-312)
    const double dphi = kPi * (3.0 - std::sqrt(5.0)), dz = 2 / static_cast<double>(n_i);
    const double phi = 0, z = 1 - dz / 2.0;
    const double a[3] = {std::cos(phi) * std::sqrt(1.0 - z * z), std::sin(phi) * std::sqrt(1.0 - z * z), z};
    const double b[3] = {std::cos(phi + dphi) * std::sqrt(1.0 - (z - dz) * (z - dz)),
                         std::sin(phi + dphi) * std::sqrt(1.0 - (z - dz) * (z - dz)), z - dz};
    const double t = dot3(a, b);
    return t > 1.0 ? 0.0 : std::acos(t);
}

double host_dist(const Geo& g, const double* a, const double* b)
{
    if (g.sphere) {
        const double t = dot3(a, b);
        return t > 1.0 ? 0.0 : std::acos(t);
    }
    return std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]));
}

int round_up(long long v, int m) { return (int)((v + m - 1) / m * m); }

Gauss make_gauss(const Geo& g, double A, double sigma);

// the least word w with random(1) >= A, so that random(1) < A exactly when w < wA
long long word_threshold(double A)
{
    long long lo = 0, hi = 1LL << 32;   // the answer lies in [lo, hi]
    while (lo < hi) {
        const long long mid = (lo + hi) / 2;
        if (ug::random_G(1, (uint32_t)mid) >= A)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

Gauss make_gauss(const Geo& g, double A, double sigma)
{
    Gauss q{};
    q.A = A;
    q.sigma_square = sigma * sigma;
    q.wA = word_threshold(A);
    const double inv = 1.0 / (2 * q.sigma_square), scale = kExpDist / g.model;
    q.exact = !(A > 0) || !(q.sigma_square > 0) || !(inv < 1e30) || !(scale < 1e30);
    q.logA = A > 0 ? (float)std::log(A) : 0.f;
    q.scale = (float)scale;
    q.inv2s2 = q.exact ? 0.f : (float)inv;
    q.rel = (float)(g.sphere ? 0.02 + 8e-7 / (g.too_close * std::sin(g.too_close)) : 0.02 + 2e-6 / g.too_close);
    return q;
}

ug_status generate(ug_ctx* ctx, const ug_topology_params& p, int n_ra, int n_i, int n_tr, uint64_t seed,
                   uint32_t net, ug_topology& t)
{
    if (p.arrangement != UG_ARRANGEMENT_SPHERE && p.arrangement != UG_ARRANGEMENT_SQUARE)
        return terr(UG_EINVAL, "unknown arrangement");
    if (n_ra <= 0 || n_i <= 0 || n_tr < 0 || n_tr > n_ra) return terr(UG_EINVAL, "bad network sizes");
    if ((long long)n_ra * n_i >= (1LL << 31)) return terr(UG_EINVAL, "N_RA * N_I must stay below 2^31");
    Geo g{};
    g.sphere = p.arrangement == UG_ARRANGEMENT_SPHERE;
    g.root = std::sqrt((double)n_i);
    g.side = (int)g.root;
    g.model = model_distance(p.arrangement, n_i);
    if (!(g.model > 0.0) || !std::isfinite(g.model))
        return terr(UG_EINVAL, "no model interneuron distance for this N_I (the sphere needs N_I >= 2)");
    g.too_close = g.model * kMinDist / kExpDist;
    if (g.sphere) {
        const double c = std::cos(g.too_close);
        g.lo = c - 1e-9;
        g.hi = c + 1e-9;
        g.lo32 = (float)(c - 2e-6);
        g.hi32 = (float)(c + 2e-6);
    } else {
        g.lo = g.too_close * g.too_close * (1 - 1e-9);
        g.hi = g.too_close * g.too_close * (1 + 1e-9);
        g.lo32 = (float)((g.too_close - 1e-6) * (g.too_close - 1e-6));
        g.hi32 = (float)((g.too_close + 1e-6) * (g.too_close + 1e-6));
    }
    g.seed = seed;
    g.net = net;
    t.params = p;
    t.n_ra = n_ra;
    t.n_i = n_i;
    t.n_tr = n_tr;
    t.model = g.model;

    TCUDA(cudaSetDevice(ug_ctx_device(ctx)));
    cudaStream_t st = ug_ctx_stream(ctx);
    Scratch mem(st);
    double *ra = nullptr, *ii = nullptr, *base = nullptr, *cand = nullptr;
    float4 *ra32 = nullptr, *ii32 = nullptr, *cand32 = nullptr;
    int *flag = nullptr, *part = nullptr, *npart = nullptr;
    State* dst = nullptr;
    TCUDA(mem.get(&ra, 3 * (size_t)n_ra));
    TCUDA(mem.get(&ii, 3 * (size_t)n_i));
    TCUDA(mem.get(&ra32, n_ra));
    TCUDA(mem.get(&ii32, n_i));
    TCUDA(mem.get(&cand32, kMaxBatch));
    TCUDA(mem.get(&base, 2 * (size_t)n_i));
    TCUDA(mem.get(&cand, 3 * (size_t)kMaxBatch));
    TCUDA(mem.get(&flag, kMaxBatch));
    TCUDA(mem.get(&npart, kMaxBatch));
    TCUDA(mem.get(&part, (size_t)kMaxBatch * kMaxPartners));
    TCUDA(mem.get(&dst, 1));
    struct Events {
        cudaEvent_t e[4] = {nullptr, nullptr, nullptr, nullptr};
        ~Events()
        {
            for (cudaEvent_t x : e)
                if (x) cudaEventDestroy(x);
        }
    } ev;
    for (cudaEvent_t& x : ev.e) TCUDA(cudaEventCreate(&x));
    cudaEvent_t ev0 = ev.e[0], ev_i = ev.e[1], ev_p = ev.e[2], ev1 = ev.e[3];
    int64_t launches = 0;
    TCUDA(cudaEventRecord(ev0, st));
    TCUDA(cudaMemsetAsync(dst, 0, sizeof(State), st));
    TCUDA(cudaMemsetAsync(ii, 0, 3 * sizeof(double) * (size_t)n_i, st));
    if (g.sphere) {
        // the Fibonacci lattice (:296-300), accumulated in the reference's order
        std::vector<double> lattice(2 * (size_t)n_i);
        const double dphi = kPi * (3.0 - std::sqrt(5.0)), dz = 2 / static_cast<double>(n_i);
        double phi = 0, z = 1 - dz / 2.0;
        for (int i = 0; i < n_i; ++i) {
            lattice[2 * i] = z;
            lattice[2 * i + 1] = phi;
            z = z - dz;
            phi = phi + dphi;
        }
        TCUDA(cudaMemcpyAsync(base, lattice.data(), lattice.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    k_i_first_tries<<<(n_i + 255) / 256, 256, 0, st>>>(g, n_i, base, ii, ii32, dst);
    ++launches;
    if (g.sphere) {
        k_i_scan<<<(n_i + kRowThreads / 32 - 1) / (kRowThreads / 32), kRowThreads, 0, st>>>(g, n_i, ii, ii32, dst);
        k_interneurons<<<1, 1024, 0, st>>>(g, n_i, ii, ii32, base, dst);
        launches += 2;
    }
    TCUDA(cudaGetLastError());
    TCUDA(cudaEventRecord(ev_i, st));

    // HVC(RA) placement in batches; an attempt meets about one conflict inside its batch
    const double pair = g.sphere ? (1 - std::cos(g.too_close)) / 2
                                 : kPi * g.too_close * g.too_close /
                                       ((1.0 - 1.0 / (g.root + 1)) * (1.0 - 1.0 / (g.root + 1)));
    int kmax = kMinBatch;
    while (kmax * 2 <= kMaxBatch && kmax * 2 * pair <= 1.0) kmax *= 2;
    int K = std::min(kmax, std::max(kMinBatch, round_up(n_ra, kMinBatch)));
    long long a0 = 0;
    State h{};
    while (h.count < n_ra) {
        if (a0 + K > 0xffffffffLL) return terr(UG_EINVAL, "HVC(RA) placement ran out of attempt streams");
        const dim3 g1((K + kCheckThreads - 1) / kCheckThreads);
        k_ra_candidates<<<g1, kCheckThreads, 0, st>>>(g, (uint32_t)a0, K, cand, cand32, flag, npart);
        const dim3 g2(g1.x, (n_i + h.count + kChunk - 1) / kChunk);
        k_ra_check_fixed<<<g2, kCheckThreads, 0, st>>>(g, cand, cand32, K, ii, ii32, n_i, ra, ra32, h.count, flag);
        const dim3 g3(g1.x, (K + kChunk - 1) / kChunk);
        k_ra_check_batch<<<g3, kCheckThreads, 0, st>>>(g, cand, cand32, K, flag, part, npart, dst);
        k_ra_resolve<<<1, kResolveThreads, 0, st>>>(cand, cand32, K, flag, part, npart, n_ra, (uint32_t)a0, ra, ra32,
                                                    dst);
        launches += 4;
        TCUDA(cudaGetLastError());
        TCUDA(cudaMemcpyAsync(&h, dst, sizeof(State), cudaMemcpyDeviceToHost, st));
        TCUDA(cudaStreamSynchronize(st));
        ++t.batches;
        if (h.status) return terr(UG_EINVAL, "interneuron placement gave up: no room at the minimum distance");
        if (h.overflow) {   // too many conflicts inside the batch: the same attempts again, fewer at a time
            if (K == kMinBatch)
                return terr(UG_EINVAL, "HVC(RA) placement: too many close attempts in a batch");
            K = std::max(kMinBatch, K / 4);
            TCUDA(cudaMemsetAsync(&dst->overflow, 0, sizeof(int), st));
            continue;
        }
        a0 += K;
        if (h.count < n_ra && a0 - h.last_kept > kMaxMisses)
            return terr(UG_EINVAL, "HVC(RA) placement gave up after " + std::to_string(a0 - h.last_kept) +
                                       " attempts in a row too close to a placed neuron (no room at the minimum "
                                       "intersomatic distance)");
        // next batch: the attempts still needed at the last batch's keep rate, with a margin, and
        // about kmax attempts left open by the points already placed
        const double rate = std::max((double)h.kept / K, 1.0 / 64);
        const double open = std::max((double)h.unflagged / K, 1.0 / 64);
        const int limit = std::min(kMaxBatch, std::max(kMinBatch, round_up((long long)(kmax / open), kMinBatch)));
        K = std::min(limit, std::max(kMinBatch, round_up((long long)((n_ra - h.count) / rate * 1.25) + 1, kMinBatch)));
    }
    t.ra_attempts = h.attempts;
    t.i_retries = h.retries;
    TCUDA(cudaEventRecord(ev_p, st));

    // connections: decide, count, scan, fill (RA->I with A_RA2I, I->RA with B_I2RA)
    const int nw_ri = (n_i + 31) / 32, nw_ir = (n_ra + 31) / 32;
    unsigned *bits_ri = nullptr, *bits_ir = nullptr;
    int *cnt_ri = nullptr, *cnt_ir = nullptr, *off_ri = nullptr, *off_ir = nullptr;
    TCUDA(mem.get(&bits_ri, (size_t)n_ra * nw_ri));
    TCUDA(mem.get(&bits_ir, (size_t)n_i * nw_ir));
    TCUDA(mem.get(&cnt_ri, n_ra));
    TCUDA(mem.get(&cnt_ir, n_i));
    TCUDA(mem.get(&off_ri, n_ra + 1));
    TCUDA(mem.get(&off_ir, n_i + 1));
    const int rows = kRowThreads / 32;
    const Gauss q_ri = make_gauss(g, p.A_RA2I, p.SIGMA_RA2I), q_ir = make_gauss(g, p.B_I2RA, p.SIGMA_I2RA);
    k_conn_decide<<<(n_ra + rows - 1) / rows, kRowThreads, 0, st>>>(g, q_ri, ra, ra32, n_ra, ii, ii32, n_i, kPartRA2I,
                                                                   bits_ri, nw_ri, cnt_ri);
    k_conn_decide<<<(n_i + rows - 1) / rows, kRowThreads, 0, st>>>(g, q_ir, ii, ii32, n_i, ra, ra32, n_ra, kPartI2RA,
                                                                  bits_ir, nw_ir, cnt_ir);
    k_scan<<<1, 1024, 0, st>>>(cnt_ri, n_ra, off_ri);
    k_scan<<<1, 1024, 0, st>>>(cnt_ir, n_i, off_ir);
    launches += 4;
    TCUDA(cudaGetLastError());
    int totals[2] = {0, 0};
    TCUDA(cudaMemcpyAsync(totals, off_ri + n_ra, sizeof(int), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaMemcpyAsync(totals + 1, off_ir + n_i, sizeof(int), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaStreamSynchronize(st));
    int *tgt_ri = nullptr, *tgt_ir = nullptr;
    double *len_ri = nullptr, *len_ir = nullptr;
    TCUDA(mem.get(&tgt_ri, totals[0]));
    TCUDA(mem.get(&tgt_ir, totals[1]));
    TCUDA(mem.get(&len_ri, totals[0]));
    TCUDA(mem.get(&len_ir, totals[1]));
    k_conn_fill<<<(n_ra + rows - 1) / rows, kRowThreads, 0, st>>>(g, ra, n_ra, ii, bits_ri, nw_ri, off_ri, tgt_ri,
                                                                 len_ri);
    k_conn_fill<<<(n_i + rows - 1) / rows, kRowThreads, 0, st>>>(g, ii, n_i, ra, bits_ir, nw_ir, off_ir, tgt_ir,
                                                                len_ir);
    launches += 2;
    TCUDA(cudaGetLastError());
    TCUDA(cudaEventRecord(ev1, st));
    t.ra_xyz.resize(3 * (size_t)n_ra);
    t.i_xyz.resize(3 * (size_t)n_i);
    t.ri_off.resize(n_ra + 1);
    t.ir_off.resize(n_i + 1);
    t.ri_tgt.resize(totals[0]);
    t.ri_len.resize(totals[0]);
    t.ir_tgt.resize(totals[1]);
    t.ir_len.resize(totals[1]);
    TCUDA(cudaMemcpyAsync(t.ra_xyz.data(), ra, t.ra_xyz.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaMemcpyAsync(t.i_xyz.data(), ii, t.i_xyz.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaMemcpyAsync(t.ri_off.data(), off_ri, t.ri_off.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaMemcpyAsync(t.ir_off.data(), off_ir, t.ir_off.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaMemcpyAsync(t.ri_tgt.data(), tgt_ri, t.ri_tgt.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaMemcpyAsync(t.ri_len.data(), len_ri, t.ri_len.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaMemcpyAsync(t.ir_tgt.data(), tgt_ir, t.ir_tgt.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaMemcpyAsync(t.ir_len.data(), len_ir, t.ir_len.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    TCUDA(cudaStreamSynchronize(st));
    TCUDA(cudaEventElapsedTime(&t.device_ms, ev0, ev1));
    TCUDA(cudaEventElapsedTime(&t.stage_ms[0], ev0, ev_i));
    TCUDA(cudaEventElapsedTime(&t.stage_ms[1], ev_i, ev_p));
    TCUDA(cudaEventElapsedTime(&t.stage_ms[2], ev_p, ev1));
    t.launches = launches;
    ug_ctx_add_launches(ctx, launches);

    // training arrangements (:406-457): neuron 0 with its nearest neighbours, then a random set
    t.clustered.assign(n_tr, 0);
    t.random_set.assign(n_tr, 0);
    if (n_tr > 0) {
        std::vector<double> d(n_ra - 1);
        for (int i = 1; i < n_ra; ++i) d[i - 1] = host_dist(g, &t.ra_xyz[0], &t.ra_xyz[3 * (size_t)i]);
        // the n_tr - 1 nearest, in order of distance (ties by index)
        std::vector<int> idx(d.size());
        std::iota(idx.begin(), idx.end(), 0);
        std::partial_sort(idx.begin(), idx.begin() + (n_tr - 1), idx.end(),
                          [&d](int a, int b) { return d[a] < d[b] || (d[a] == d[b] && a < b); });
        for (int i = 1; i < n_tr; ++i) t.clustered[i] = idx[i - 1] + 1;
        std::vector<int> unsampled(n_ra);
        std::iota(unsampled.begin(), unsampled.end(), 0);
        ug::HostStream hs{ug::make_stream(seed, ug::kNoiseTopology, net, 0, kPartTraining), 0};
        for (int i = 0; i < n_tr; ++i) {
            // sample_integer(0, N_RA - i - 1)
            const int k = (int)(((uint64_t)hs.word() * (uint64_t)(n_ra - i)) >> 32);
            t.random_set[i] = unsampled[k];
            unsampled[k] = unsampled.back();
            unsampled.pop_back();
        }
    }
    return UG_OK;
}

}  // namespace

extern "C" {

ug_status ug_generate_topology(ug_ctx* ctx, const ug_topology_params* params, int32_t n_ra, int32_t n_i,
                               int32_t n_tr, uint64_t seed, int32_t stream_id, ug_topology** out)
{
    if (!ctx || !params || !out) return terr(UG_EINVAL, "null argument");
    *out = nullptr;
    std::lock_guard<std::recursive_mutex> lk(ug_ctx_mutex(ctx));
    ug_topology* t = new ug_topology();
    const ug_status s = generate(ctx, *params, n_ra, n_i, n_tr, seed, (uint32_t)stream_id, *t);
    if (s != UG_OK) {
        delete t;
        return s;
    }
    *out = t;
    return UG_OK;
}

ug_status ug_topology_get_info(const ug_topology* t, ug_topology_info* info)
{
    if (!t || !info) return terr(UG_EINVAL, "null argument");
    std::memset(info, 0, sizeof(*info));
    info->n_ra = t->n_ra;
    info->n_i = t->n_i;
    info->n_tr = t->n_tr;
    info->dim = t->dim();
    info->n_ra2i = (int64_t)t->ri_tgt.size();
    info->n_i2ra = (int64_t)t->ir_tgt.size();
    info->ra_attempts = t->ra_attempts;
    info->i_retries = t->i_retries;
    info->model_distance = t->model;
    info->device_ms = t->device_ms;
    info->interneuron_ms = t->stage_ms[0];
    info->placement_ms = t->stage_ms[1];
    info->connection_ms = t->stage_ms[2];
    info->batches = t->batches;
    info->launches = t->launches;
    return UG_OK;
}

ug_status ug_topology_get_coordinates(const ug_topology* t, double* ra_xyz, double* i_xyz)
{
    if (!t) return terr(UG_EINVAL, "null topology");
    if (ra_xyz) std::copy(t->ra_xyz.begin(), t->ra_xyz.end(), ra_xyz);
    if (i_xyz) std::copy(t->i_xyz.begin(), t->i_xyz.end(), i_xyz);
    return UG_OK;
}

ug_status ug_topology_get_connections(const ug_topology* t, int32_t which, int32_t* offsets, int32_t* targets,
                                      double* lengths)
{
    if (!t || (which != 0 && which != 1)) return terr(UG_EINVAL, "bad topology or connection kind");
    const std::vector<int32_t>& off = which == 0 ? t->ri_off : t->ir_off;
    const std::vector<int32_t>& tgt = which == 0 ? t->ri_tgt : t->ir_tgt;
    const std::vector<double>& len = which == 0 ? t->ri_len : t->ir_len;
    if (offsets) std::copy(off.begin(), off.end(), offsets);
    if (targets) std::copy(tgt.begin(), tgt.end(), targets);
    if (lengths) std::copy(len.begin(), len.end(), lengths);
    return UG_OK;
}

ug_status ug_topology_get_training(const ug_topology* t, int32_t which, int32_t* neurons)
{
    if (!t || (which != 0 && which != 1) || !neurons) return terr(UG_EINVAL, "bad topology or training kind");
    const std::vector<int32_t>& v = which == 0 ? t->clustered : t->random_set;
    std::copy(v.begin(), v.end(), neurons);
    return UG_OK;
}

void ug_topology_free(ug_topology* t) { delete t; }

}  // extern "C"
