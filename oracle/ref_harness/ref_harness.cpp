/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * C entry points around the reference's own HVC(RA) and HVC(I) classes
 * (c++/src/HH2_test.cpp, c++/src/HHI_buffer.cpp, compiled unmodified from the
 * reference tree into oracle/_ref by oracle/Makefile).  They step one neuron
 * with the trial path's per-step call (Debraband_step_no_target_update,
 * HH2_test.cpp:535-545; DP8_step_no_target_update, HHI_buffer.cpp:332-339)
 * and record its state, so the oracle's restatement can be pinned to the
 * reference's arithmetic.  Signatures match ugo_ra_single / ugo_i_single.
 */
#include "poisson_noise.h"
#include "HH2_test.h"
#include "HHI_buffer.h"
#include <cstring>
#include <cstdint>

namespace {

struct ProbeRA : public HH2_test {
    void row(double* out) const
    {
        double r[10] = { _Vs, _Vd, _n, _h, _l, _r, _c, _Ca, _Gexc_d, _Ginh_d };
        std::memcpy(out, r, sizeof(r));
    }
    bool soma() const { return _fired_soma; }
    bool dend() const { return _fired_dend; }
};

struct ProbeI : public HHI_buffer {
    void row(double* out) const
    {
        double r[7] = { _voltage, _n, _m, _h, _w, _Gexc, _Ginh };
        std::memcpy(out, r, sizeof(r));
    }
    bool fired() const { return _fired; }
};

struct NoiseParams {
    double white_noise_mean_soma, white_noise_std_soma, white_noise_mean_dend, white_noise_std_dend;
};

} // namespace

extern "C" void ref_ra_single(int32_t n_steps, double Erest, double GCa, const NoiseParams* noise,
                              uint64_t seed, uint32_t trial, uint32_t neuron, const int32_t* kick_step,
                              const double* kick_exc, const double* kick_inh, int32_t n_kicks,
                              double* trace_out, uint8_t* fired_out)
{
    Poisson_noise gen;
    gen.bind(seed, UGO_KIND_RA_WHITE, 0, neuron, trial);
    ProbeRA n;
    n.set_noise_generator(&gen);
    n.set_white_noise(noise->white_noise_mean_soma, noise->white_noise_std_soma,
                      noise->white_noise_mean_dend, noise->white_noise_std_dend);
    n.set_dynamics(0.02);
    n.set_Erest(Erest);
    n.set_GCa(GCa);
    int kk = 0;
    for (int t = 0; t < n_steps; ++t) {
        while (kk < n_kicks && kick_step[kk] == t) {
            n.raiseE(kick_exc[kk]);
            n.raiseI(kick_inh[kk]);
            ++kk;
        }
        n.Debraband_step_no_target_update();
        n.row(trace_out + (size_t)t * 10);
        fired_out[2 * t] = n.soma() ? 1 : 0;
        fired_out[2 * t + 1] = n.dend() ? 1 : 0;
    }
}

extern "C" void ref_i_single(int32_t n_steps, uint64_t seed, uint32_t trial, uint32_t neuron,
                             const int32_t* kick_step, const double* kick_exc, const double* kick_inh,
                             int32_t n_kicks, double* trace_out, uint8_t* fired_out)
{
    Poisson_noise gen;
    gen.bind(seed, UGO_KIND_I_POISSON, 0, neuron, trial);
    ProbeI n;
    n.set_noise_generator(&gen);
    n.set_dynamics(0.02);
    n.set_poisson_noise();
    int kk = 0;
    for (int t = 0; t < n_steps; ++t) {
        while (kk < n_kicks && kick_step[kk] == t) {
            n.raiseE(kick_exc[kk]);
            n.raiseI(kick_inh[kk]);
            ++kk;
        }
        n.DP8_step_no_target_update();
        n.row(trace_out + (size_t)t * 7);
        fired_out[t] = n.fired() ? 1 : 0;
    }
}
