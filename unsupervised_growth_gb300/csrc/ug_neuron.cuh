// Neuron integrators of the trial path, one neuron per thread.
//
//  * HVC(RA): two-compartment Hodgkin-Huxley neuron (c++/include/HH2_test.h,
//    c++/src/HH2_test.cpp) advanced by the 4-stage Debrabant weak-order-3
//    stochastic Runge-Kutta step with 30-point noise (HH2_test.cpp:613-754).
//  * HVC(I): single-compartment interneuron (c++/include/HHI_buffer.h,
//    c++/src/HHI_buffer.cpp) advanced by the 12-stage Dormand-Prince 8 step
//    (HHI_buffer.cpp:426-690) with Poisson conductance noise.
//
// The double instantiation follows the reference's operation order term by
// term (the translation unit is compiled without multiply-add contraction), so
// it reproduces the reference's double-precision results up to the last-bit
// differences of the device exp().  The float instantiation computes the same
// equations with SFU exponentials and merged reciprocals (8 ex2 + 7 rcp per RA
// stage, 7 ex2 + 4 rcp per I stage).
//
// RA somatic conductances are not carried: on the trial path HVC(RA) neurons
// get no Poisson noise (set_noise, NetworkGrowthSimulator.cpp:2061-2075) and
// every kick goes to the dendrite, so Gexc_s = Ginh_s = 0 throughout.
#pragma once
#include <stdint.h>
#include "ug_philox.cuh"

namespace ug {

// ---------------------------------------------------------------- constants
// HH2_test.cpp:262-289 and thresholds HH2_test.cpp:25-28
struct RAConst {
    static constexpr double cm = 1.0, As = 5000.0, Ad = 10000.0, Rc = 55.0;
    static constexpr double GsKLT = 3.5, GsK = 8.0, GsNa = 60.0, GdCaK = 150.0, GsL = 0.1, GdL = 0.1;
    static constexpr double EdCa = 120.0, EdK = -90.0, EsNa = 55.0, EsK = -90.0, Egaba = -80.0;
    static constexpr double tau = 5.0;  // tExc = tInh
};
// HHI_buffer.cpp:13-37
struct IConst {
    static constexpr double cm = 1.0, A = 6000.0;
    static constexpr double Ena = 55.0, Ek = -80.0, El = -65.0, Ei = -75.0;
    static constexpr double gNa = 100.0, gKdr = 20.0, gKHT = 500.0, gL = 0.1;
    static constexpr double tExc = 2.0, tInh = 5.0;
    static constexpr double G_noise = 0.45, lambda = 250.0;
};

template <class R>
struct RAState {
    R Vs, Vd, n, h, l, r, c, Ca, Ge, Gi;
};

template <class R>
struct IStateR {
    R V, n, m, h, w, Ge, Gi;
};

// Per-step inputs of the RA step that do not depend on the neuron.
template <class R>
struct RAStep {
    R dt, sq;             // dt and sqrt(dt)
    R sig_s, sig_d;       // white-noise amplitudes
    R mu_s, mu_d;         // white-noise means
    R e1, e2;             // conductance decay to t+dt and t+dt/2 (exp(-h/5))
    uint32_t ks[20];      // the network's Philox key schedule (k0, k1 of rounds 0..9), for the packed kernel
};

// Philox4x32-10 key schedule of a seed: (k0, k1) of each of the ten rounds.
inline void philox_key_schedule(uint64_t seed, uint32_t* ks)
{
    uint32_t k0 = (uint32_t)(seed & 0xffffffffu), k1 = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        ks[2 * r] = k0;
        ks[2 * r + 1] = k1;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

__device__ __forceinline__ double ra_point(int idx, double)
{
    const double s6 = 2.449489742783178098197284;  // sqrt(6) (the reference computes sqrt(6) in double)
    return idx == 0 ? s6 : idx == 1 ? -s6 : idx <= 10 ? 1.0 : idx <= 19 ? -1.0 : 0.0;
}
__device__ __forceinline__ float ra_point(int idx, float)
{
    const float s6 = 2.4494897f;
    return idx == 0 ? s6 : idx == 1 ? -s6 : idx <= 10 ? 1.0f : idx <= 19 ? -1.0f : 0.0f;
}

// ------------------------------------------------------------ RA, double
struct RAKd { double Vs, Vd, n, l, h, r, c, Ca; };

__device__ __forceinline__ RAKd ra_rhs_d(double vs, double vd, double n, double h, double l, double r, double c,
                                        double ca, double Ge_d, double Gi_d, double EL, double GdCa, double mu_s,
                                        double mu_d)
{
    typedef RAConst K;
    RAKd k;
    const double m = 1 / (1 + exp(-(vs + 30) / 9.5));
    const double m3 = m * m * m;
    const double n4 = n * n * n * n;
    k.Vs = (-K::GsL * (vs - EL) - K::GsNa * m3 * h * (vs - K::EsNa) - K::GsK * n4 * (vs - K::EsK)
            - K::GsKLT * l * (vs - K::EsK) + 100000 * (0.0 + mu_s) / K::As + 100000 * (vd - vs) / (K::Rc * K::As)) / K::cm;
    const double r2 = r * r;
    k.Vd = (-K::GdL * (vd - EL) - GdCa * r2 * (vd - K::EdCa) - K::GdCaK * (vd - K::EdK) * c / (1 + 6 / ca)
            - Ge_d * vd - Gi_d * (vd - K::Egaba) + 100000 * (0.0 + mu_d) / K::Ad + 100000 * (vs - vd) / (K::Rc * K::Ad)) / K::cm;
    k.n = (1 / (1 + exp(-(vs + 35) / 10)) - n) / (0.1 + 0.5 / (1 + exp((vs + 27) / 15)));
    k.l = (1 / (1 + exp(-(vs + 40) / 5)) - l) / 10.0;
    k.h = (1 / (1 + exp((vs + 45) / 7)) - h) / (0.1 + 0.75 / (1 + exp((vs + 40.5) / 6)));
    k.r = (1 / (1 + exp(-(vd + 5) / 10)) - r) / 1;
    k.c = (1 / (1 + exp(-(vd - 10) / 7)) - c) / 15;
    k.Ca = (-0.1 * GdCa * r * r * (vd - K::EdCa) - 0.02 * ca);
    return k;
}

__device__ __forceinline__ void ra_debrabant(RAState<double>& s, double EL, double GdCa, const RAStep<double>& p,
                                             double J1s, double J2s, double J1d, double J2d)
{
    typedef RAConst K;
    const double dt = p.dt, sq = p.sq;
    const double H1Vs = s.Vs + sq * p.sig_s * (-0.01844540496323970 * J1s - 0.1866426386543421 * J2s) / (K::As * K::cm);
    const double H1Vd = s.Vd + sq * p.sig_d * (-0.01844540496323970 * J1d - 0.1866426386543421 * J2d) / (K::Ad * K::cm);
    const RAKd a1 = ra_rhs_d(H1Vs, H1Vd, s.n, s.h, s.l, s.r, s.c, s.Ca, s.Ge, s.Gi, EL, GdCa, p.mu_s, p.mu_d);

    const double Ge1 = s.Ge * p.e1, Gi1 = s.Gi * p.e1, Ge2 = s.Ge * p.e2, Gi2 = s.Gi * p.e2;
    const double H2Vs = s.Vs + dt * a1.Vs + sq * p.sig_s * (0.8017012756521233 * J1s - 0.8575745885712401 * J2s) / (K::As * K::cm);
    const double H2Vd = s.Vd + dt * a1.Vd + sq * p.sig_d * (0.8017012756521233 * J1d - 0.8575745885712401 * J2d) / (K::Ad * K::cm);
    const RAKd a2 = ra_rhs_d(H2Vs, H2Vd, s.n + dt * a1.n, s.h + dt * a1.h, s.l + dt * a1.l, s.r + dt * a1.r,
                             s.c + dt * a1.c, s.Ca + dt * a1.Ca, Ge1, Gi1, EL, GdCa, p.mu_s, p.mu_d);

    const double H3Vs = s.Vs + dt * (3 * a1.Vs + a2.Vs) / 8 + sq * p.sig_s * (0.5092227024816198 * J1s - 0.4723392695015512 * J2s) / (K::As * K::cm);
    const double H3Vd = s.Vd + dt * (3 * a1.Vd + a2.Vd) / 8 + sq * p.sig_d * (0.5092227024816198 * J1d - 0.4723392695015512 * J2d) / (K::Ad * K::cm);
    const RAKd a3 = ra_rhs_d(H3Vs, H3Vd, s.n + dt * (3 * a1.n + a2.n) / 8, s.h + dt * (3 * a1.h + a2.h) / 8,
                             s.l + dt * (3 * a1.l + a2.l) / 8, s.r + dt * (3 * a1.r + a2.r) / 8,
                             s.c + dt * (3 * a1.c + a2.c) / 8, s.Ca + dt * (3 * a1.Ca + a2.Ca) / 8, Ge2, Gi2, EL, GdCa,
                             p.mu_s, p.mu_d);

    const double b1 = -0.4526683126055039, b2 = -0.4842227708685013, b3 = 1.9368910834740051;
    const double H4Vs = s.Vs + dt * (b1 * a1.Vs + b2 * a2.Vs + b3 * a3.Vs)
                        + sq * p.sig_s * (0.9758794209767762 * J1s + 0.3060354860326548 * J2s) / (K::As * K::cm);
    const double H4Vd = s.Vd + dt * (b1 * a1.Vd + b2 * a2.Vd + b3 * a3.Vd)
                        + sq * p.sig_d * (0.9758794209767762 * J1d + 0.3060354860326548 * J2d) / (K::Ad * K::cm);
    const RAKd a4 = ra_rhs_d(H4Vs, H4Vd, s.n + dt * (b1 * a1.n + b2 * a2.n + b3 * a3.n),
                             s.h + dt * (b1 * a1.h + b2 * a2.h + b3 * a3.h), s.l + dt * (b1 * a1.l + b2 * a2.l + b3 * a3.l),
                             s.r + dt * (b1 * a1.r + b2 * a2.r + b3 * a3.r), s.c + dt * (b1 * a1.c + b2 * a2.c + b3 * a3.c),
                             s.Ca + dt * (b1 * a1.Ca + b2 * a2.Ca + b3 * a3.Ca), Ge1, Gi1, EL, GdCa, p.mu_s, p.mu_d);

    const double q2 = 0.005430430675258792, q4 = 0.1720970973419255;
    s.Vs = s.Vs + dt * (a1.Vs / 6 - q2 * a2.Vs + 2 * a3.Vs / 3 + q4 * a4.Vs) + sq * p.sig_s * J1s * 100000 / (K::As * K::cm);
    s.Vd = s.Vd + dt * (a1.Vd / 6 - q2 * a2.Vd + 2 * a3.Vd / 3 + q4 * a4.Vd) + sq * p.sig_d * J1d * 100000 / (K::Ad * K::cm);
    s.Ca = s.Ca + dt * (a1.Ca / 6 - q2 * a2.Ca + 2 * a3.Ca / 3 + q4 * a4.Ca);
    s.n = s.n + dt * (a1.n / 6 - q2 * a2.n + 2 * a3.n / 3 + q4 * a4.n);
    s.l = s.l + dt * (a1.l / 6 - q2 * a2.l + 2 * a3.l / 3 + q4 * a4.l);
    s.h = s.h + dt * (a1.h / 6 - q2 * a2.h + 2 * a3.h / 3 + q4 * a4.h);
    s.r = s.r + dt * (a1.r / 6 - q2 * a2.r + 2 * a3.r / 3 + q4 * a4.r);
    s.c = s.c + dt * (a1.c / 6 - q2 * a2.c + 2 * a3.c / 3 + q4 * a4.c);
    s.Ge = s.Ge * p.e1;
    s.Gi = s.Gi * p.e1;
}

// ------------------------------------------------------------- RA, float
struct RAKf { float Vs, Vd, n, l, h, r, c, Ca; };

__device__ __forceinline__ float fexp(float x) { return __expf(x); }
__device__ __forceinline__ float frcp(float x) { return __fdividef(1.0f, x); }

__device__ __forceinline__ RAKf ra_rhs_f(float vs, float vd, float n, float h, float l, float r, float c, float ca,
                                        float Ge_d, float Gi_d, float EL, float GdCa, float mu_term_s, float mu_term_d)
{
    typedef RAConst K;
    RAKf k;
    const float m = frcp(1.0f + fexp((vs + 30.0f) * (-1.0f / 9.5f)));
    const float m3 = m * m * m;
    const float n2 = n * n;
    const float n4 = n2 * n2;
    const float coup_s = (vd - vs) * (float)(100000.0 / (K::Rc * K::As));
    k.Vs = -(float)K::GsL * (vs - EL) - (float)K::GsNa * m3 * h * (vs - (float)K::EsNa)
           - ((float)K::GsK * n4 + (float)K::GsKLT * l) * (vs - (float)K::EsK) + mu_term_s + coup_s;
    // GdCaK (vd - EdK) c / (1 + 6/ca) = GdCaK (vd - EdK) c ca / (ca + 6)
    const float cak = (float)K::GdCaK * (vd - (float)K::EdK) * c * ca * frcp(ca + 6.0f);
    k.Vd = -(float)K::GdL * (vd - EL) - GdCa * r * r * (vd - (float)K::EdCa) - cak - Ge_d * vd
           - Gi_d * (vd - (float)K::Egaba) + mu_term_d + (vs - vd) * (float)(100000.0 / (K::Rc * K::Ad));
    // kn = (nInf - n) / tauN with nInf = 1/(1+En), tauN = 0.1 + 0.5/(1+Et): one reciprocal
    {
        const float En = fexp((vs + 35.0f) * -0.1f);
        const float Et = fexp((vs + 27.0f) * (1.0f / 15.0f));
        const float a = 1.0f + En, b = 1.0f + Et;
        k.n = (1.0f - n * a) * b * frcp(a * (0.1f * b + 0.5f));
    }
    k.l = (frcp(1.0f + fexp((vs + 40.0f) * -0.2f)) - l) * 0.1f;
    {
        const float Eh = fexp((vs + 45.0f) * (1.0f / 7.0f));
        const float Et = fexp((vs + 40.5f) * (1.0f / 6.0f));
        const float a = 1.0f + Eh, b = 1.0f + Et;
        k.h = (1.0f - h * a) * b * frcp(a * (0.1f * b + 0.75f));
    }
    k.r = frcp(1.0f + fexp((vd + 5.0f) * -0.1f)) - r;
    k.c = (frcp(1.0f + fexp((vd - 10.0f) * (-1.0f / 7.0f))) - c) * (1.0f / 15.0f);
    k.Ca = (-0.1f * GdCa) * r * r * (vd - (float)K::EdCa) - 0.02f * ca;
    return k;
}

__device__ __forceinline__ void ra_debrabant(RAState<float>& s, float EL, float GdCa, const RAStep<float>& p,
                                             float J1s, float J2s, float J1d, float J2d)
{
    typedef RAConst K;
    const float dt = p.dt;
    const float ns = p.sq * p.sig_s * (float)(1.0 / (K::As * K::cm));
    const float nd = p.sq * p.sig_d * (float)(1.0 / (K::Ad * K::cm));
    const float mus = (float)(100000.0 / K::As) * p.mu_s, mud = (float)(100000.0 / K::Ad) * p.mu_d;
    const float Ge1 = s.Ge * p.e1, Gi1 = s.Gi * p.e1, Ge2 = s.Ge * p.e2, Gi2 = s.Gi * p.e2;

    const RAKf a1 = ra_rhs_f(s.Vs + ns * (-0.01844540496323970f * J1s - 0.1866426386543421f * J2s),
                             s.Vd + nd * (-0.01844540496323970f * J1d - 0.1866426386543421f * J2d), s.n, s.h, s.l, s.r,
                             s.c, s.Ca, s.Ge, s.Gi, EL, GdCa, mus, mud);
    const RAKf a2 = ra_rhs_f(s.Vs + dt * a1.Vs + ns * (0.8017012756521233f * J1s - 0.8575745885712401f * J2s),
                             s.Vd + dt * a1.Vd + nd * (0.8017012756521233f * J1d - 0.8575745885712401f * J2d),
                             s.n + dt * a1.n, s.h + dt * a1.h, s.l + dt * a1.l, s.r + dt * a1.r, s.c + dt * a1.c,
                             s.Ca + dt * a1.Ca, Ge1, Gi1, EL, GdCa, mus, mud);
    const float d8 = dt * 0.125f;
    const RAKf a3 = ra_rhs_f(s.Vs + d8 * (3.0f * a1.Vs + a2.Vs) + ns * (0.5092227024816198f * J1s - 0.4723392695015512f * J2s),
                             s.Vd + d8 * (3.0f * a1.Vd + a2.Vd) + nd * (0.5092227024816198f * J1d - 0.4723392695015512f * J2d),
                             s.n + d8 * (3.0f * a1.n + a2.n), s.h + d8 * (3.0f * a1.h + a2.h), s.l + d8 * (3.0f * a1.l + a2.l),
                             s.r + d8 * (3.0f * a1.r + a2.r), s.c + d8 * (3.0f * a1.c + a2.c), s.Ca + d8 * (3.0f * a1.Ca + a2.Ca),
                             Ge2, Gi2, EL, GdCa, mus, mud);
    const float b1 = -0.4526683126055039f, b2 = -0.4842227708685013f, b3 = 1.9368910834740051f;
#define UG_H4(f) (s.f + dt * (b1 * a1.f + b2 * a2.f + b3 * a3.f))
    const RAKf a4 = ra_rhs_f(UG_H4(Vs) + ns * (0.9758794209767762f * J1s + 0.3060354860326548f * J2s),
                             UG_H4(Vd) + nd * (0.9758794209767762f * J1d + 0.3060354860326548f * J2d), UG_H4(n), UG_H4(h),
                             UG_H4(l), UG_H4(r), UG_H4(c), UG_H4(Ca), Ge1, Gi1, EL, GdCa, mus, mud);
#undef UG_H4
    const float q1 = 1.0f / 6.0f, q2 = -0.005430430675258792f, q3 = 2.0f / 3.0f, q4 = 0.1720970973419255f;
#define UG_UPD(f) (s.f + dt * (q1 * a1.f + q2 * a2.f + q3 * a3.f + q4 * a4.f))
    s.Vs = UG_UPD(Vs) + ns * 100000.0f * J1s;
    s.Vd = UG_UPD(Vd) + nd * 100000.0f * J1d;
    s.Ca = UG_UPD(Ca);
    s.n = UG_UPD(n);
    s.l = UG_UPD(l);
    s.h = UG_UPD(h);
    s.r = UG_UPD(r);
    s.c = UG_UPD(c);
#undef UG_UPD
    s.Ge = Ge1;
    s.Gi = Gi1;
}

// Spike detection on the state before the step (HH2_test::state_check,
// HH2_test.cpp:561-594).  flags bit0 = soma flag, bit1 = dendrite flag.
template <class R>
__device__ __forceinline__ void ra_state_check(const RAState<R>& s, int& flags, bool& fired_soma, bool& fired_dend)
{
    const int fs = flags & 1, fd = (flags >> 1) & 1;
    int nfs = fs, nfd = fd;
    fired_soma = false;
    fired_dend = false;
    if (fs == 1 && s.Vs < R(-35.0)) {
        nfs = 0;
        fired_soma = true;
    } else if (fs == 0 && s.Vs > R(-30.0)) {
        nfs = 1;
    }
    if (fd == 0 && s.Vd >= R(-30.0)) {
        nfd = 1;
        fired_dend = true;
    } else if (fd == 1 && s.Vd < R(-35.0)) {
        nfd = 0;
    }
    flags = (flags & ~3) | nfs | (nfd << 1);
}

// One trial-path RA step: check, draw the step's 4 point indices (block
// `step-1` of the neuron's stream, in the order ind1s, ind2s, ind1d, ind2d,
// HH2_test.cpp:640-643), integrate.
template <class R>
__device__ __forceinline__ void ra_step(RAState<R>& s, int& flags, bool& fired_soma, bool& fired_dend, R EL, R GdCa,
                                        const RAStep<R>& p, const StreamId& sid, uint32_t step)
{
    ra_state_check(s, flags, fired_soma, fired_dend);
    const Philox4 w = stream_block(sid, step - 1);
    ra_debrabant(s, EL, GdCa, p, ra_point(point_index(w.x), R(0)), ra_point(point_index(w.y), R(0)),
                 ra_point(point_index(w.z), R(0)), ra_point(point_index(w.w), R(0)));
}

// -------------------------------------------------------------- I, DP8
// Butcher tableau of the reference's DP8 step (HHI_buffer.cpp:426-690).
// Stages 2..6: x + dt * (sum of small integer multiples of k) / den.
// Stages 7..12 and the update: x + dt * sum(num * k / den).
struct DPT { int s; double num, den; };

#define UG_DP_B7 {0, 29443841, 614563906}, {3, 77736538, 692538347}, {4, -28693883, 1125000000}, {5, 23124283, 1800000000}
#define UG_DP_B8 {0, 16016141, 946692911}, {3, 61564180, 158732637}, {4, 22789713, 633445777}, \
                 {5, 545815736, 2771057229.0}, {6, -180193667, 1043307555}
#define UG_DP_B9 {0, 39632708, 573591083}, {3, -433636366, 683701615}, {4, -421739975, 2616292301.0}, \
                 {5, 100302831, 723423059}, {6, 790204164, 839813087}, {7, 800635310, 3783071287.0}
#define UG_DP_B10 {0, 246121993, 1340847787}, {3, -37695042795.0, 15268766246.0}, {4, -309121744, 1061227803}, \
                  {5, -12992083, 490766935}, {6, 6005943493.0, 2108947869}, {7, 393006217, 1396673457}, \
                  {8, 123872331, 1001029789}
#define UG_DP_B11 {0, -1028468189, 846180014}, {3, 8478235783.0, 508512852}, {4, 1311729495, 1432422823}, \
                  {5, -10304129995.0, 1701304382}, {6, -48777925059.0, 3047939560.0}, {7, 15336726248.0, 1032824649}, \
                  {8, -45442868181.0, 3398467696.0}, {9, 3065993473.0, 597172653}
#define UG_DP_B12 {0, 185892177, 718116043}, {3, -3185094517.0, 667107341}, {4, -477755414, 1098053517}, \
                  {5, -703635378, 230739211}, {6, 5731566787.0, 1027545527}, {7, 5232866602.0, 850066563}, \
                  {8, -4093664535.0, 808688257}, {9, 3962137247.0, 1805957418}, {10, 65686358, 487910083}
#define UG_DP_OUT {0, 13451932, 455176623}, {5, -808719846, 976000145}, {6, 1757004468, 5645159321.0}, \
                  {7, 656045339, 265891186}, {8, -3867574721.0, 1518517206}, {9, 465885868, 322736535}, \
                  {10, 53011238, 667516719}, {11, 2, 45}

// stage time offsets as num * dt / den (stage 1 has none)
#define UG_DP_CNUM 0, 1, 1, 1, 5, 3, 59, 93, 5490023248.0, 13, 1201146811, 1
#define UG_DP_CDEN 1, 18, 12, 8, 16, 8, 400, 200, 9719169821.0, 20, 12990119798.0, 1

// Per-step conductance decay factors of the 12 stages and the update:
// ge[k] = exp(-h_k / tExc), gi[k] = exp(-h_k / tInh), h_k = stage time - step start.
template <class R>
struct IStep {
    R dt;
    R ge[12], gi[12];   // index 0 is stage 1 (factor 1); index 11 is also the update's factor
};

struct IKd { double V, n, m, h, w; };

__device__ __forceinline__ IKd i_rhs_d(double v, double h, double w, double m3, double n4, double n, double m, double Ge,
                                       double Gi)
{
    typedef IConst K;
    IKd k;
    k.V = (-K::gL * (v - K::El) - K::gNa * h * m3 * (v - K::Ena) - K::gKdr * n4 * (v - K::Ek)
           - K::gKHT * w * (v - K::Ek) - Ge * v - Gi * (v - K::Ei) + 100000 * 0.0 / K::A) / K::cm;
    k.n = 0.15 * (v + 15) / (1 - exp(-(v + 15) / 10)) * (1 - n) - 0.2 * exp(-(v + 25) / 80) * n;
    k.m = (v + 22) / (1 - exp(-(v + 22) / 10)) * (1 - m) - 40 * exp(-(v + 47) / 18) * m;
    k.h = 0.7 * exp(-(v + 34) / 20) * (1 - h) - 10 / (1 + exp(-(v + 4) / 10)) * h;
    k.w = (1 / (1 + exp(-v / 5)) - w) / 1;
    return k;
}

struct IKf { float V, n, m, h, w; };

// x / (1 - exp(-x/10)) with its removable singularity at x = 0 handled by the series 10 (1 + x/20 + x^2/1200)
__device__ __forceinline__ float i_vtrap(float x)
{
    if (fabsf(x) < 1e-3f) return 10.0f + x * (0.5f + x * (1.0f / 120.0f));
    return __fdividef(x, 1.0f - __expf(x * -0.1f));
}

__device__ __forceinline__ IKf i_rhs_f(float v, float h, float w, float m3, float n4, float n, float m, float Ge, float Gi)
{
    typedef IConst K;
    IKf k;
    k.V = -(float)K::gL * (v - (float)K::El) - (float)K::gNa * h * m3 * (v - (float)K::Ena)
          - ((float)K::gKdr * n4 + (float)K::gKHT * w) * (v - (float)K::Ek) - Ge * v - Gi * (v - (float)K::Ei);
    k.n = 0.15f * i_vtrap(v + 15.0f) * (1.0f - n) - 0.2f * __expf((v + 25.0f) * (-1.0f / 80.0f)) * n;
    k.m = i_vtrap(v + 22.0f) * (1.0f - m) - 40.0f * __expf((v + 47.0f) * (-1.0f / 18.0f)) * m;
    k.h = 0.7f * __expf((v + 34.0f) * -0.05f) * (1.0f - h) - 10.0f * __fdividef(h, 1.0f + __expf((v + 4.0f) * -0.1f));
    k.w = __fdividef(1.0f, 1.0f + __expf(v * -0.2f)) - w;
    return k;
}

template <class R>
__device__ __forceinline__ void i_dp8(IStateR<R>& s, const IStep<R>& p);

template <>
__device__ __forceinline__ void i_dp8<double>(IStateR<double>& s, const IStep<double>& p)
{
    const DPT B7[] = {UG_DP_B7}, B8[] = {UG_DP_B8}, B9[] = {UG_DP_B9}, B10[] = {UG_DP_B10}, B11[] = {UG_DP_B11},
              B12[] = {UG_DP_B12}, BO[] = {UG_DP_OUT};
    const DPT* tb[6] = {B7, B8, B9, B10, B11, B12};
    const int cnt[6] = {4, 5, 6, 7, 8, 9};
    const int acount[5] = {1, 2, 2, 3, 3};
    const int astage[5][3] = {{0, 0, 0}, {0, 1, 0}, {0, 2, 0}, {0, 2, 3}, {0, 3, 4}};
    const double acoef[5][3] = {{1, 0, 0}, {1, 3, 0}, {1, 3, 0}, {20, -75, 75}, {3, 15, 12}};
    const double aden[5] = {18, 48, 32, 64, 80};
    const double dt = p.dt;
    double kV[12], kn[12], km[12], kh[12], kw[12];
#pragma unroll
    for (int st = 0; st < 12; ++st) {
        double v, n1, m1, h1, w1;
        if (st == 0) {
            v = s.V; n1 = s.n; m1 = s.m; h1 = s.h; w1 = s.w;
        } else if (st <= 5) {
            const int a = st - 1;
            double sV = acoef[a][0] * kV[astage[a][0]], sn = acoef[a][0] * kn[astage[a][0]],
                   sm = acoef[a][0] * km[astage[a][0]], sh = acoef[a][0] * kh[astage[a][0]],
                   sw = acoef[a][0] * kw[astage[a][0]];
#pragma unroll
            for (int j = 1; j < 3; ++j) {
                if (j < acount[a]) {
                    const int q = astage[a][j];
                    const double c = acoef[a][j];
                    sV = sV + c * kV[q]; sn = sn + c * kn[q]; sm = sm + c * km[q]; sh = sh + c * kh[q]; sw = sw + c * kw[q];
                }
            }
            m1 = s.m + dt * sm / aden[a];
            n1 = s.n + dt * sn / aden[a];
            h1 = s.h + dt * sh / aden[a];
            w1 = s.w + dt * sw / aden[a];
            v = s.V + dt * sV / aden[a];
        } else {
            const DPT* t = tb[st - 6];
            const int c = cnt[st - 6];
            double sV = t[0].num * kV[t[0].s] / t[0].den, sn = t[0].num * kn[t[0].s] / t[0].den,
                   sm = t[0].num * km[t[0].s] / t[0].den, sh = t[0].num * kh[t[0].s] / t[0].den,
                   sw = t[0].num * kw[t[0].s] / t[0].den;
#pragma unroll
            for (int j = 1; j < 9; ++j) {
                if (j < c) {
                    const int q = t[j].s;
                    sV = sV + t[j].num * kV[q] / t[j].den;
                    sn = sn + t[j].num * kn[q] / t[j].den;
                    sm = sm + t[j].num * km[q] / t[j].den;
                    sh = sh + t[j].num * kh[q] / t[j].den;
                    sw = sw + t[j].num * kw[q] / t[j].den;
                }
            }
            m1 = s.m + dt * sm;
            n1 = s.n + dt * sn;
            h1 = s.h + dt * sh;
            w1 = s.w + dt * sw;
            v = s.V + dt * sV;
        }
        const double n4 = n1 * n1 * n1 * n1;
        const double m3 = m1 * m1 * m1;
        const IKd k = i_rhs_d(v, h1, w1, m3, n4, n1, m1, s.Ge * p.ge[st], s.Gi * p.gi[st]);
        kV[st] = k.V; kn[st] = k.n; km[st] = k.m; kh[st] = k.h; kw[st] = k.w;
    }
    double oV = BO[0].num * kV[BO[0].s] / BO[0].den, on = BO[0].num * kn[BO[0].s] / BO[0].den,
           om = BO[0].num * km[BO[0].s] / BO[0].den, oh = BO[0].num * kh[BO[0].s] / BO[0].den,
           ow = BO[0].num * kw[BO[0].s] / BO[0].den;
#pragma unroll
    for (int j = 1; j < 8; ++j) {
        const int q = BO[j].s;
        oV = oV + BO[j].num * kV[q] / BO[j].den;
        on = on + BO[j].num * kn[q] / BO[j].den;
        om = om + BO[j].num * km[q] / BO[j].den;
        oh = oh + BO[j].num * kh[q] / BO[j].den;
        ow = ow + BO[j].num * kw[q] / BO[j].den;
    }
    s.V = s.V + dt * oV;
    s.n = s.n + dt * on;
    s.m = s.m + dt * om;
    s.h = s.h + dt * oh;
    s.w = s.w + dt * ow;
    s.Ge = s.Ge * p.ge[11];
    s.Gi = s.Gi * p.gi[11];
}

template <>
__device__ __forceinline__ void i_dp8<float>(IStateR<float>& s, const IStep<float>& p)
{
    // Same tableau; coefficients folded to num/den in float at compile time.
    const DPT B7[] = {UG_DP_B7}, B8[] = {UG_DP_B8}, B9[] = {UG_DP_B9}, B10[] = {UG_DP_B10}, B11[] = {UG_DP_B11},
              B12[] = {UG_DP_B12}, BO[] = {UG_DP_OUT};
    const DPT* tb[6] = {B7, B8, B9, B10, B11, B12};
    const int cnt[6] = {4, 5, 6, 7, 8, 9};
    const int acount[5] = {1, 2, 2, 3, 3};
    const int astage[5][3] = {{0, 0, 0}, {0, 1, 0}, {0, 2, 0}, {0, 2, 3}, {0, 3, 4}};
    const double acoef[5][3] = {{1, 0, 0}, {1, 3, 0}, {1, 3, 0}, {20, -75, 75}, {3, 15, 12}};
    const double aden[5] = {18, 48, 32, 64, 80};
    const float dt = p.dt;
    float kV[12], kn[12], km[12], kh[12], kw[12];
#pragma unroll
    for (int st = 0; st < 12; ++st) {
        float v, n1, m1, h1, w1;
        if (st == 0) {
            v = s.V; n1 = s.n; m1 = s.m; h1 = s.h; w1 = s.w;
        } else {
            float sV = 0.f, sn = 0.f, sm = 0.f, sh = 0.f, sw = 0.f;
            if (st <= 5) {
                const int a = st - 1;
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    if (j < acount[a]) {
                        const int q = astage[a][j];
                        const float c = (float)(acoef[a][j] / aden[a]);
                        sV += c * kV[q]; sn += c * kn[q]; sm += c * km[q]; sh += c * kh[q]; sw += c * kw[q];
                    }
                }
            } else {
                const DPT* t = tb[st - 6];
#pragma unroll
                for (int j = 0; j < 9; ++j) {
                    if (j < cnt[st - 6]) {
                        const int q = t[j].s;
                        const float c = (float)(t[j].num / t[j].den);
                        sV += c * kV[q]; sn += c * kn[q]; sm += c * km[q]; sh += c * kh[q]; sw += c * kw[q];
                    }
                }
            }
            v = s.V + dt * sV;
            n1 = s.n + dt * sn;
            m1 = s.m + dt * sm;
            h1 = s.h + dt * sh;
            w1 = s.w + dt * sw;
        }
        const float n2 = n1 * n1;
        const IKf k = i_rhs_f(v, h1, w1, m1 * m1 * m1, n2 * n2, n1, m1, s.Ge * p.ge[st], s.Gi * p.gi[st]);
        kV[st] = k.V; kn[st] = k.n; km[st] = k.m; kh[st] = k.h; kw[st] = k.w;
    }
    float oV = 0.f, on = 0.f, om = 0.f, oh = 0.f, ow = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int q = BO[j].s;
        const float c = (float)(BO[j].num / BO[j].den);
        oV += c * kV[q]; on += c * kn[q]; om += c * km[q]; oh += c * kh[q]; ow += c * kw[q];
    }
    s.V = s.V + dt * oV;
    s.n = s.n + dt * on;
    s.m = s.m + dt * om;
    s.h = s.h + dt * oh;
    s.w = s.w + dt * ow;
    s.Ge = s.Ge * p.ge[11];
    s.Gi = s.Gi * p.gi[11];
}

// Interneuron spike detection (HHI_buffer::state_check, HHI_buffer.cpp:260-276).
template <class R>
__device__ __forceinline__ bool i_state_check(R V, int& flag)
{
    if (flag == 1 && V < R(-25.0)) {
        flag = 0;
        return true;
    }
    if (flag == 0 && V > R(-20.0)) flag = 1;
    return false;
}

// Poisson conductance noise (HHI_buffer::noise_check, HHI_buffer.cpp:278-294);
// time is the neuron's time at the start of the step.
__device__ __forceinline__ void i_noise_check(double time, double dt, double& G, double& noise_time, const StreamId& sid,
                                              uint32_t& word)
{
    if (time > noise_time) {
        G += random_G(IConst::G_noise, stream_word(sid, word++));
        double rnd = 1000 * (-log(1 - u01(stream_word(sid, word++))) / IConst::lambda);
        while (rnd < dt) {
            rnd = 1000 * (-log(1 - u01(stream_word(sid, word++))) / IConst::lambda);
            G += random_G(IConst::G_noise, stream_word(sid, word++));
        }
        noise_time = noise_time + rnd;
    }
}

// First noisy-spike time (HHI_buffer::initialize_noise, HHI_buffer.cpp:217-239).
__device__ __forceinline__ double i_initial_noise_time(const StreamId& sid, uint32_t& word, double dt)
{
    double t = 1000 * (-log(1 - u01(stream_word(sid, word++))) / IConst::lambda);
    while (t < dt) t = 1000 * (-log(1 - u01(stream_word(sid, word++))) / IConst::lambda);
    return t;
}

}  // namespace ug
