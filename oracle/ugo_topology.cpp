/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- see ug_oracle.h.
 *
 * Sequential CPU restatement of the reference's network topology generation
 * (createNetworkForGrowth: NetworkGrowthSimulator::generate_network_topology,
 * c++/src/NetworkGrowthSimulator.cpp:110-155), the checker for the device
 * generator of the product library.
 *
 *   sample_coordinates            :222-403  Fibonacci-sphere interneurons with
 *                                           jitter, uniform HVC(RA) on the sphere,
 *                                           both with rejection on the minimum
 *                                           intersomatic distance; or the square
 *                                           grid arrangement
 *   sample_connections            :620-705  Gaussian-probability RA->I, I->RA
 *   p_RA2I, p_I2RA                :707-719
 *   write_different_training_arrangements :406-457  clustered and random sets
 *
 * The reference draws from its rank's mt19937 in program order.  Here every
 * draw comes from a counter-based stream of kind UGO_KIND_TOPOLOGY, one per
 * purpose, so that the device generator can make the same draws in parallel:
 *   trial field 0, entity i : interneuron i, words 2r, 2r+1 for its r-th try
 *                             (theta then phi jitter; x then y on the square)
 *   trial field 1, entity a : the a-th HVC(RA) placement attempt, words 0, 1
 *                             (z then phi; x then y on the square)
 *   trial field 2, entity i : RA->I row i, word j decides the pair (i, j)
 *   trial field 3, entity i : I->RA row i, word j decides the pair (i, j)
 *   trial field 4, entity 0 : the random training arrangement, sequential words
 * The RA placement keeps the reference's semantics exactly: attempt a is
 * accepted when it is far enough from every interneuron and from every HVC(RA)
 * accepted before it, and the next neuron continues with attempt a + 1.
 * The sample_G(0.0) draw of each new connection is not made (its value is 0).
 * Where the reference would loop for ever (no room left at the minimum distance),
 * both give up once one neuron has been rejected max_misses times in a row.
 */
#include "ug_oracle.h"
#include "ugo_noise.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace {

const double kPi = 3.14159265358979323846;
const double kExperimentalInterneuronDistance = 40.0;   /* NetworkGrowthSimulator.cpp:19 */
const double kMinIntersomaticDistance = 10.0;           /* NetworkGrowthSimulator.cpp:20 */
const double kNoiseShift = 0.15;                        /* sample_coordinates :224 */

/* distance_on_sphere (NetworkGrowthSimulator.cpp:36-44) and distance2d (:31-34) */
double dist_sphere(const double* a, const double* b)
{
    const double tmp = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    return tmp > 1.0 ? 0.0 : std::acos(tmp);
}

double dist_square(const double* a, const double* b)
{
    return std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]));
}

struct Gen {
    const ugo_topology_params* p;
    int n_ra, n_i;
    uint64_t seed;
    uint32_t net;
    bool sphere;
    double model, too_close;

    double dist(const double* a, const double* b) const { return sphere ? dist_sphere(a, b) : dist_square(a, b); }

    void word2(uint32_t part, uint32_t entity, uint32_t first, uint32_t* u) const
    {
        ugo_stream s;
        ugo_stream_init(&s, seed, UGO_KIND_TOPOLOGY, net, entity, part);
        for (uint32_t k = 0; k < first; ++k) ugo_stream_word(&s);
        u[0] = ugo_stream_word(&s);
        u[1] = ugo_stream_word(&s);
    }
};

}  // namespace

extern "C" double ugo_topology_model_distance(int32_t arrangement, int32_t n_i)
{
    if (arrangement == 1) return 1 / (std::sqrt((double)n_i) + 1);
    /* the first two points of the Fibonacci lattice (:296-312) */
    const double dphi = kPi * (3.0 - std::sqrt(5.0));
    const double dz = 2 / static_cast<double>(n_i);
    const double phi = 0, z = 1 - dz / 2.0;
    const double a[3] = {std::cos(phi) * std::sqrt(1.0 - z * z), std::sin(phi) * std::sqrt(1.0 - z * z), z};
    const double b[3] = {std::cos(phi + dphi) * std::sqrt(1.0 - (z - dz) * (z - dz)),
                         std::sin(phi + dphi) * std::sqrt(1.0 - (z - dz) * (z - dz)), z - dz};
    return dist_sphere(a, b);
}

extern "C" int ugo_generate_topology(const ugo_topology_params* p, int32_t n_ra, int32_t n_i, int32_t n_tr,
                                     uint64_t seed, uint32_t net, int64_t max_misses, double* ra_xyz,
                                     double* i_xyz, double* model_out, int32_t* ri_off, int32_t* ri_tgt,
                                     double* ri_len, int64_t ri_cap, int32_t* ir_off, int32_t* ir_tgt,
                                     double* ir_len, int64_t ir_cap, int32_t* clustered, int32_t* random_tr,
                                     int64_t* counters)
{
    if (n_ra <= 0 || n_i <= 0 || n_tr < 0 || n_tr > n_ra) return -3;
    Gen g{p, n_ra, n_i, seed, net, p->arrangement == 0, 0.0, 0.0};
    g.model = ugo_topology_model_distance(p->arrangement, n_i);
    g.too_close = g.model * kMinIntersomaticDistance / kExperimentalInterneuronDistance;
    *model_out = g.model;
    std::fill(ra_xyz, ra_xyz + 3 * (size_t)n_ra, 0.0);
    std::fill(i_xyz, i_xyz + 3 * (size_t)n_i, 0.0);
    int64_t i_retries = 0, attempts = 0;
    uint32_t u[2];

    if (g.sphere) {
        /* interneurons: Fibonacci lattice, jittered, rejected when too close to an earlier one */
        const double dphi = kPi * (3.0 - std::sqrt(5.0));
        const double dz = 2 / static_cast<double>(n_i);
        double phi = 0, z = 1 - dz / 2.0;
        for (int i = 0; i < n_i; ++i) {
            double t[3];
            bool too_close = true;
            for (uint32_t r = 0; too_close; ++r) {
                if (r > (uint32_t)max_misses) return -1;
                if (r > 0) ++i_retries;
                too_close = false;
                g.word2(0, (uint32_t)i, 2 * r, u);
                const double theta = std::acos(z);
                const double theta_noise = -kNoiseShift * g.model + ugo_random_G(2 * kNoiseShift * g.model, u[0]);
                const double phi_noise =
                    (-kNoiseShift * g.model + ugo_random_G(2 * kNoiseShift * g.model, u[1])) / std::sin(theta);
                t[0] = std::cos(phi + phi_noise) * std::sin(theta + theta_noise);
                t[1] = std::sin(phi + phi_noise) * std::sin(theta + theta_noise);
                t[2] = std::cos(theta + theta_noise);
                for (int j = 0; j < i; ++j)
                    if (dist_sphere(t, i_xyz + 3 * j) < g.too_close) {
                        too_close = true;
                        break;
                    }
            }
            std::copy(t, t + 3, i_xyz + 3 * i);
            z = z - dz;
            phi = phi + dphi;
        }
    } else {
        /* square grid of floor(sqrt(N_I))^2 interneurons; the rest stay at the origin (:231-241) */
        const int s = (int)std::sqrt((double)n_i);
        const double root = std::sqrt((double)n_i);
        for (int i = 0; i < s; ++i)
            for (int k = 0; k < s; ++k) {
                const int q = i * s + k;
                g.word2(0, (uint32_t)q, 0, u);
                i_xyz[3 * q] = (double)(i + 1) / (root + 1) - kNoiseShift * g.model +
                               ugo_random_G(2 * kNoiseShift * g.model, u[0]);
                i_xyz[3 * q + 1] = (double)(k + 1) / (root + 1) - kNoiseShift * g.model +
                                   ugo_random_G(2 * kNoiseShift * g.model, u[1]);
            }
    }

    /* HVC(RA): uniform attempts, rejected when too close to any interneuron or earlier HVC(RA) */
    const double root = std::sqrt((double)n_i);
    for (int i = 0; i < n_ra; ++i) {
        double t[3] = {0, 0, 0};
        bool too_close = true;
        for (int64_t misses = 0; too_close; ++misses) {
            if (misses > max_misses || attempts >= 0xffffffffLL) return -1;
            g.word2(1, (uint32_t)attempts, 0, u);
            ++attempts;
            if (g.sphere) {
                const double zz = 2 * ugo_random_G(1.0, u[0]) - 1;
                const double ph = ugo_random_G(2.0 * kPi, u[1]);
                t[0] = std::sin(std::acos(zz)) * std::cos(ph);
                t[1] = std::sin(std::acos(zz)) * std::sin(ph);
                t[2] = zz;
            } else {
                t[0] = 0.5 / (root + 1) + ugo_random_G(1.0 - 1.0 / (root + 1), u[0]);
                t[1] = 0.5 / (root + 1) + ugo_random_G(1.0 - 1.0 / (root + 1), u[1]);
            }
            too_close = false;
            for (int j = 0; j < n_i && !too_close; ++j) too_close = g.dist(t, i_xyz + 3 * j) < g.too_close;
            for (int j = 0; j < i && !too_close; ++j) too_close = g.dist(t, ra_xyz + 3 * j) < g.too_close;
        }
        std::copy(t, t + 3, ra_xyz + 3 * i);
    }

    /* connections: RA->I rows then I->RA rows, each pair decided by its own word */
    auto connect = [&](const double* src, int n_src, const double* dst, int n_dst, uint32_t part, double A,
                       double sigma, int32_t* off, int32_t* tgt, double* len, int64_t cap) {
        const double sigma_square = sigma * sigma;
        int64_t e = 0;
        off[0] = 0;
        for (int i = 0; i < n_src; ++i) {
            ugo_stream s;
            ugo_stream_init(&s, seed, UGO_KIND_TOPOLOGY, net, (uint32_t)i, part);
            for (int j = 0; j < n_dst; ++j) {
                const double d = g.dist(src + 3 * i, dst + 3 * j) * kExperimentalInterneuronDistance / g.model;
                if (ugo_random_G(1, ugo_stream_word(&s)) < A * std::exp(-d * d / (2 * sigma_square))) {
                    if (e >= cap) return false;
                    tgt[e] = j;
                    len[e] = d;
                    ++e;
                }
            }
            off[i + 1] = (int32_t)e;
        }
        return true;
    };
    if (!connect(ra_xyz, n_ra, i_xyz, n_i, 2, p->A_RA2I, p->SIGMA_RA2I, ri_off, ri_tgt, ri_len, ri_cap)) return -2;
    if (!connect(i_xyz, n_i, ra_xyz, n_ra, 3, p->B_I2RA, p->SIGMA_I2RA, ir_off, ir_tgt, ir_len, ir_cap)) return -2;

    /* training arrangements: neuron 0 with its nearest neighbours, then a random set */
    if (n_tr > 0) {
        std::vector<double> d(n_ra - 1);
        for (int i = 1; i < n_ra; ++i) d[i - 1] = g.dist(ra_xyz, ra_xyz + 3 * i);
        std::vector<int> idx(d.size());
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&d](int a, int b) { return d[a] < d[b]; });
        clustered[0] = 0;
        for (int i = 1; i < n_tr; ++i) clustered[i] = idx[i - 1] + 1;
        std::vector<int> unsampled(n_ra);
        std::iota(unsampled.begin(), unsampled.end(), 0);
        ugo_stream s;
        ugo_stream_init(&s, seed, UGO_KIND_TOPOLOGY, net, 0, 4);
        for (int i = 0; i < n_tr; ++i) {
            /* sample_integer(0, N_RA - i - 1) */
            const int k = (int)(((uint64_t)ugo_stream_word(&s) * (uint64_t)(n_ra - i)) >> 32);
            random_tr[i] = unsampled[k];
            unsampled[k] = unsampled.back();
            unsampled.pop_back();
        }
    }
    counters[0] = attempts;
    counters[1] = i_retries;
    return 0;
}
