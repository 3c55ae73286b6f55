// ug_growth: the reference's four programs on the GB300 engine, with their argument
// lists (c++/createNetworkForGrowth/main.cpp, c++/chainGrowth/main.cpp,
// c++/continueChainGrowth/main.cpp, c++/chainTest/main.cpp) and their output files.
//
//   ug_growth createNetworkForGrowth <topology config> <network dir>
//   ug_growth chainGrowth <network dir> <training neurons file> <growth config> <output dir>
//   ug_growth continueChainGrowth <data dir> <output dir> <starting trial>
//   ug_growth chainTest <network dir> <trial number> <number of test trials> <output dir>
//
// Options (after the positional arguments): --trials N (growth trials to run; the
// reference runs until stopped), --save-short K, --save-long K (the reference's
// save frequencies: 75/150 for chainGrowth, 50/100 for continueChainGrowth),
// --precision 32|64, --device D, --seed S (noise streams; 15000 by default),
// --spike-capacity C (spikes recorded per neuron and trial for the spike files);
// createNetworkForGrowth takes --n-ra, --n-i, --n-tr (2000, 550 and 10, the sizes its
// reference main hard-codes), --seed and --device.  --track-inhibition R (ms) makes the
// growth programs run the inhibition-tracking variant (new_chain_growth_with_inhibition_tracking,
// NetworkGrowthSimulator.cpp:1784-1862): every trial records each HVC(RA) neuron's Ginh_d every
// R ms and writes write_inhibition_tracking_state's files; the full state every --save-long trials.
//
// Growth saves are written after a trial's between-trial bookkeeping, so
// continueChainGrowth from a saved trial T runs trials T + 1, T + 2, ...
#include "ugrowth.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct Opts {
    long trials = -1;
    int save_short = -1, save_long = -1, precision = 32, device = 0, spikes = 256;
    int n_ra = 2000, n_i = 550, n_tr = 10;
    double track = 0.0;   // inhibition tracking resolution (ms), 0: off
    unsigned long long seed = 15000;
};

bool parse_opts(int argc, char** argv, int first, Opts& o)
{
    for (int i = first; i < argc; ++i) {
        const std::string a = argv[i];
        if (i + 1 >= argc) {
            std::fprintf(stderr, "option %s needs a value\n", a.c_str());
            return false;
        }
        const char* v = argv[++i];
        if (a == "--trials") o.trials = std::atol(v);
        else if (a == "--save-short") o.save_short = std::atoi(v);
        else if (a == "--save-long") o.save_long = std::atoi(v);
        else if (a == "--precision") o.precision = std::atoi(v);
        else if (a == "--device") o.device = std::atoi(v);
        else if (a == "--seed") o.seed = std::strtoull(v, nullptr, 10);
        else if (a == "--spike-capacity") o.spikes = std::atoi(v);
        else if (a == "--n-ra") o.n_ra = std::atoi(v);
        else if (a == "--n-i") o.n_i = std::atoi(v);
        else if (a == "--n-tr") o.n_tr = std::atoi(v);
        else if (a == "--track-inhibition") o.track = std::atof(v);
        else {
            std::fprintf(stderr, "unknown option %s\n", a.c_str());
            return false;
        }
    }
    return true;
}

int check(ug_status s, const char* what)
{
    if (s == UG_OK) return 0;
    std::fprintf(stderr, "%s: %s\n", what, ug_last_error());
    return 1;
}

std::string path(const std::string& dir, const std::string& name)
{
    return dir.empty() || dir.back() == '/' ? dir + name : dir + "/" + name;
}

// chain_growth (NetworkGrowthSimulator.cpp:5731-5845): a growth trial, then the graph
// state every save_short trials and the full state every save_long trials.
// chain_growth_with_inhibition_tracking (:5662-5729): the full state every save_long
// trials and the inhibition-tracking state after every trial.
int grow(ug_ctx* ctx, int net, long first, const Opts& o, const std::string& out)
{
    const long last = o.trials < 0 ? (1L << 30) : first + o.trials;
    if (o.track > 0 && check(ug_set_inhibition_tracking(ctx, net, o.track), "inhibition tracking")) return 1;
    for (long t = first; t < last; ++t) {
        const ug_status s = ug_run_growth_trials(ctx, net, (uint32_t)t, 1, 1);
        if (s == UG_ENUMERIC) {
            std::printf("Bad values in neuron dynamics!\n");
            return 1;
        }
        if (check(s, "growth trial")) return 1;
        std::printf("Trial %ld\n", t);
        if (o.track > 0) {
            if (t % o.save_long == 0 &&
                check(ug_write_state_dir(ctx, net, out.c_str(), ("_" + std::to_string(t)).c_str(), (int32_t)t),
                      "full state"))
                return 1;
            if (check(ug_write_inhibition_tracking_state(ctx, net, out.c_str(), (int32_t)t), "inhibition tracking state"))
                return 1;
            continue;
        }
        if (t % o.save_short == 0 && check(ug_write_graph_state(ctx, net, out.c_str(), (int32_t)t), "graph state"))
            return 1;
        if (t % o.save_long == 0 &&
            check(ug_write_state_dir(ctx, net, out.c_str(), ("_" + std::to_string(t)).c_str(), (int32_t)t),
                  "full state"))
            return 1;
    }
    return 0;
}

int usage()
{
    std::fprintf(stderr,
                 "usage:\n"
                 "  ug_growth createNetworkForGrowth <topology config> <network dir> [--n-ra N --n-i N --n-tr N]\n"
                 "  ug_growth chainGrowth <network dir> <training neurons file> <growth config> <output dir> [options]\n"
                 "  ug_growth continueChainGrowth <data dir> <output dir> <starting trial> [options]\n"
                 "  ug_growth chainTest <network dir> <trial number> <number of test trials> <output dir> [options]\n"
                 "options: --trials N --save-short K --save-long K --precision 32|64 --device D --seed S\n"
                 "         --track-inhibition R (the inhibition-tracking growth variant, Ginh_d every R ms)\n"
                 "         --spike-capacity C (spikes recorded per neuron and trial, 256 by default)\n");
    return 2;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 2) return usage();
    const std::string cmd = argv[1];
    const int npos = cmd == "chainGrowth"              ? 4
                     : cmd == "continueChainGrowth"    ? 3
                     : cmd == "chainTest"              ? 4
                     : cmd == "createNetworkForGrowth" ? 2
                                                       : -1;
    if (npos < 0 || argc < 2 + npos) return usage();
    Opts o;
    if (cmd == "continueChainGrowth") {
        o.save_short = 50;
        o.save_long = 100;
    } else {
        o.save_short = 75;
        o.save_long = 150;
    }
    if (!parse_opts(argc, argv, 2 + npos, o)) return usage();
    if (o.save_short <= 0 || o.save_long <= 0) return usage();
    ug_runtime_opts ro = {o.precision, o.device, o.spikes, 1};
    ug_ctx* ctx = nullptr;
    if (check(ug_create(&ctx, &ro), "ug_create")) return 1;
    int rc = 0;
    int32_t net = -1;
    if (cmd == "createNetworkForGrowth") {
        // generate_network_topology (NetworkGrowthSimulator.cpp:110-155)
        ug_topology_info info;
        rc = check(ug_create_network_topology(ctx, argv[2], argv[3], o.n_ra, o.n_i, o.n_tr, o.seed, &info),
                   "generate_network_topology");
        if (!rc)
            std::printf("Model interneuron distance = %g\nN_RA = %d, N_I = %d: %lld RA->I and %lld I->RA connections\n",
                        info.model_distance, info.n_ra, info.n_i, (long long)info.n_ra2i, (long long)info.n_i2ra);
    } else if (cmd == "chainGrowth") {
        const std::string out = argv[5];
        rc = check(ug_create_growth_network(ctx, argv[2], argv[3], argv[4], out.c_str(), 0, o.seed, 0, &net),
                   "network set-up");
        if (!rc) rc = grow(ctx, net, 0, o, out);
    } else if (cmd == "continueChainGrowth") {
        const long start = std::atol(argv[4]);
        rc = check(ug_load_network_dir(ctx, argv[2], (int32_t)start, 0, o.seed, 0, &net), "read_network_state");
        if (!rc) rc = grow(ctx, net, start + 1, o, argv[3]);
    } else {
        const int trial = std::atoi(argv[3]), n = std::atoi(argv[4]);
        const std::string out = argv[5];
        if (n <= 0 || n > 65535) {
            std::fprintf(stderr, "the number of test trials must lie in [1, 65535]\n");
            rc = 1;
        }
        if (!rc) rc = check(ug_load_network_dir(ctx, argv[2], trial, 0, o.seed, 0, &net), "read_network_state");
        // test_chain (NetworkGrowthSimulator.cpp:1313-1482): every trial at once, then the
        // per-trial spike files (write_chain_test) and jitter.bin
        if (!rc) rc = check(ug_run_test_trials(ctx, net, 0, n), "test trials");
        const char* kinds[] = {"soma", "dend", "interneuron"};
        for (int k = 0; k < n && !rc; ++k)
            for (int w = 0; w < 3 && !rc; ++w) {
                const std::string p = path(out, std::string("test_spike_times_") + kinds[w] + "_" + std::to_string(k) + ".bin");
                rc = check(ug_write_spike_times(ctx, net, k, w, p.c_str(), trial), "spike times");
            }
        if (!rc) rc = check(ug_write_jitter(ctx, net, path(out, "jitter.bin").c_str()), "jitter");
    }
    ug_destroy(ctx);
    return rc;
}
