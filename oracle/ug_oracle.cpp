/*
 * ORACLE / TEST INFRASTRUCTURE ONLY -- see ug_oracle.h.
 *
 * Double-precision CPU restatement of the reference's per-trial hot path.
 * Every arithmetic expression keeps the reference's operation order so that,
 * compiled with -ffp-contract=off against the same libm, the neuron
 * trajectories are bit-identical to the reference's own classes (the tests
 * check this against outputs of c++/src/HH2_test.cpp and c++/src/HHI_buffer.cpp
 * compiled under oracle/_ref).
 */
#include "ug_oracle.h"
#include "ugo_noise.h"

#include <climits>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>
#include <algorithm>
#include <utility>

namespace {

/* ------------------------------------------------------------------------ */
/* HVC(RA) two-compartment neuron: c++/src/HH2_test.cpp, c++/include/HH2_test.h */
/* ------------------------------------------------------------------------ */

/* Fixed model constants (HH2_test.cpp:262-289, thresholds HH2_test.cpp:25-28). */
const double RA_cm = 1.0, RA_As = 5000.0, RA_Ad = 10000.0, RA_Rc = 55.0;
const double RA_GsKLT = 3.5, RA_GsK = 8.0, RA_GsNa = 60.0, RA_GdCaK = 150.0;
const double RA_GsL = 0.1, RA_GdL = 0.1;
const double RA_EdCa = 120.0, RA_EdK = -90.0, RA_EsNa = 55.0, RA_EsK = -90.0, RA_Egaba = -80.0;
const double RA_tExc = 5.0, RA_tInh = 5.0;
const double RA_threshold_spike = -30.0, RA_threshold_burst = -30.0;
const double RA_spike_margin = 5.0, RA_burst_margin = 5.0;

/* 30-point distribution of the weak-order-3 scheme (HH2_test.cpp:33-35). */
double ra_point_value(int idx)
{
    if (idx == 0) return std::sqrt(6.0);
    if (idx == 1) return -std::sqrt(6.0);
    if (idx <= 10) return 1.0;
    if (idx <= 19) return -1.0;
    return 0.0;
}

struct RAState {
    double Vs, Vd, n, h, l, r, c, Ca;
    double Gexc_s, Ginh_s, Gexc_d, Ginh_d;
    double time;
    int flag_soma, flag_dend, Nspikes, Nbursts;
    bool fired_soma, fired_dend;
};

struct RAParams {
    double EL;      /* EsL = EdL (set_Erest, HH2_test.h:50) */
    double GdCa;    /* set_GCa, HH2_test.h:54 */
    double mu_s, sigma_s, mu_d, sigma_d;
    double dt;
};

/* set_to_rest, HH2_test.cpp:191-242 */
void ra_set_to_rest(RAState& s)
{
    s.time = 0.0;
    s.Vs = -79.97619025;
    s.Vd = -79.97268759;
    s.l = 0.0;
    s.n = 0.01101284;
    s.h = 0.9932845;
    s.r = 0.00055429;
    s.c = 0.00000261762353;
    s.Ca = 0.01689572;
    s.Ginh_s = 0.0; s.Gexc_s = 0.0; s.Ginh_d = 0.0; s.Gexc_d = 0.0;
    s.flag_soma = 0; s.flag_dend = 0;
    s.Nspikes = 0; s.Nbursts = 0;
    s.fired_soma = false; s.fired_dend = false;
}

/* gating functions, HH2_test.h:265-276 */
inline double ra_nInf(double v) { return 1 / (1 + std::exp(-(v + 35) / 10)); }
inline double ra_tauN(double v) { return 0.1 + 0.5 / (1 + std::exp((v + 27) / 15)); }
inline double ra_hInf(double v) { return 1 / (1 + std::exp((v + 45) / 7)); }
inline double ra_tauH(double v) { return 0.1 + 0.75 / (1 + std::exp((v + 40.5) / 6)); }
inline double ra_mInf(double v) { return 1 / (1 + std::exp(-(v + 30) / 9.5)); }
inline double ra_lInf(double v) { return 1 / (1 + std::exp(-(v + 40) / 5)); }
inline double ra_rInf(double v) { return 1 / (1 + std::exp(-(v + 5) / 10)); }
inline double ra_cInf(double v) { return 1 / (1 + std::exp(-(v - 10) / 7)); }

/* Right-hand sides at stage time t, HH2_test.cpp:861-890.  Conductances decay
 * analytically from the start of the step: G(t) = G * exp(-(t - time)/tau). */
struct RADerivs { double Vs, Vd, n, l, h, r, c, Ca; };

inline RADerivs ra_rhs(const RAState& s, const RAParams& p, double vs, double vd, double n, double h,
                       double l, double r, double c, double ca, double t)
{
    RADerivs k;
    double Gi_s = s.Ginh_s * std::exp(-(t - s.time) / RA_tInh);
    double Ge_s = s.Gexc_s * std::exp(-(t - s.time) / RA_tExc);
    double Ge_d = s.Gexc_d * std::exp(-(t - s.time) / RA_tExc);
    double Gi_d = s.Ginh_d * std::exp(-(t - s.time) / RA_tInh);
    double m = ra_mInf(vs);
    double m3 = m * m * m;
    double n4 = n * n * n * n;
    const double Is = 0.0, Id = 0.0;   /* no injected current on the trial path */
    k.Vs = (-RA_GsL * (vs - p.EL) - RA_GsNa * m3 * h * (vs - RA_EsNa) - RA_GsK * n4 * (vs - RA_EsK)
            - RA_GsKLT * l * (vs - RA_EsK) - Gi_s * (vs - RA_Egaba) - Ge_s * vs
            + 100000 * (Is + p.mu_s) / RA_As + 100000 * (vd - vs) / (RA_Rc * RA_As)) / RA_cm;
    double r2 = r * r;
    k.Vd = (-RA_GdL * (vd - p.EL) - p.GdCa * r2 * (vd - RA_EdCa) - RA_GdCaK * (vd - RA_EdK) * c / (1 + 6 / ca)
            - Ge_d * vd - Gi_d * (vd - RA_Egaba) + 100000 * (Id + p.mu_d) / RA_Ad
            + 100000 * (vs - vd) / (RA_Rc * RA_Ad)) / RA_cm;
    k.n = (ra_nInf(vs) - n) / ra_tauN(vs);
    k.l = (ra_lInf(vs) - l) / 10.0;
    k.h = (ra_hInf(vs) - h) / ra_tauH(vs);
    k.r = (ra_rInf(vd) - r) / 1;
    k.c = (ra_cInf(vd) - c) / 15;
    k.Ca = (-0.1 * p.GdCa * r * r * (vd - RA_EdCa) - 0.02 * ca);
    return k;
}

/* Spike detection on the state before the step, HH2_test.cpp:561-594. */
void ra_state_check(RAState& s)
{
    if ((s.flag_soma == 1) && (s.Vs < RA_threshold_spike - RA_spike_margin)) {
        s.flag_soma = 0;
        s.fired_soma = true;
        s.Nspikes++;
    } else {
        s.fired_soma = false;
        if ((s.flag_soma == 0) && (s.Vs > RA_threshold_spike)) s.flag_soma = 1;
    }
    if ((s.flag_dend == 0) && (s.Vd >= RA_threshold_burst)) {
        s.flag_dend = 1;
        s.fired_dend = true;
        s.Nbursts++;
    } else {
        s.fired_dend = false;
        if ((s.flag_dend == 1) && (s.Vd < RA_threshold_burst - RA_burst_margin)) s.flag_dend = 0;
    }
}

/* Debrabant weak-order-3 stochastic Runge-Kutta step, HH2_test.cpp:613-754.
 * J1s, J2s, J1d, J2d are the four point-distribution values of the step.  The
 * stage noise terms lack the 100000 factor of the final update, as in the
 * reference (HH2_test.cpp:653-654 vs 729-733). */
void ra_debrabant(RAState& s, const RAParams& p, double J1s, double J2s, double J1d, double J2d)
{
    const double dt = p.dt;
    const double sq = std::sqrt(dt);
    double H1Vs = s.Vs + sq * p.sigma_s * (-0.01844540496323970 * J1s - 0.1866426386543421 * J2s) / (RA_As * RA_cm);
    double H1Vd = s.Vd + sq * p.sigma_d * (-0.01844540496323970 * J1d - 0.1866426386543421 * J2d) / (RA_Ad * RA_cm);
    RADerivs a1 = ra_rhs(s, p, H1Vs, H1Vd, s.n, s.h, s.l, s.r, s.c, s.Ca, s.time);

    double H2Vs = s.Vs + dt * a1.Vs + sq * p.sigma_s * (0.8017012756521233 * J1s - 0.8575745885712401 * J2s) / (RA_As * RA_cm);
    double H2Vd = s.Vd + dt * a1.Vd + sq * p.sigma_d * (0.8017012756521233 * J1d - 0.8575745885712401 * J2d) / (RA_Ad * RA_cm);
    RADerivs a2 = ra_rhs(s, p, H2Vs, H2Vd, s.n + dt * a1.n, s.h + dt * a1.h, s.l + dt * a1.l,
                         s.r + dt * a1.r, s.c + dt * a1.c, s.Ca + dt * a1.Ca, s.time + dt);

    double H3Vs = s.Vs + dt * (3 * a1.Vs + a2.Vs) / 8 + sq * p.sigma_s * (0.5092227024816198 * J1s - 0.4723392695015512 * J2s) / (RA_As * RA_cm);
    double H3Vd = s.Vd + dt * (3 * a1.Vd + a2.Vd) / 8 + sq * p.sigma_d * (0.5092227024816198 * J1d - 0.4723392695015512 * J2d) / (RA_Ad * RA_cm);
    RADerivs a3 = ra_rhs(s, p, H3Vs, H3Vd, s.n + dt * (3 * a1.n + a2.n) / 8, s.h + dt * (3 * a1.h + a2.h) / 8,
                         s.l + dt * (3 * a1.l + a2.l) / 8, s.r + dt * (3 * a1.r + a2.r) / 8,
                         s.c + dt * (3 * a1.c + a2.c) / 8, s.Ca + dt * (3 * a1.Ca + a2.Ca) / 8, s.time + 0.5 * dt);

    const double b1 = -0.4526683126055039, b2 = -0.4842227708685013, b3 = 1.9368910834740051;
    double H4Vs = s.Vs + dt * (b1 * a1.Vs + b2 * a2.Vs + b3 * a3.Vs)
                  + sq * p.sigma_s * (0.9758794209767762 * J1s + 0.3060354860326548 * J2s) / (RA_As * RA_cm);
    double H4Vd = s.Vd + dt * (b1 * a1.Vd + b2 * a2.Vd + b3 * a3.Vd)
                  + sq * p.sigma_d * (0.9758794209767762 * J1d + 0.3060354860326548 * J2d) / (RA_Ad * RA_cm);
    RADerivs a4 = ra_rhs(s, p, H4Vs, H4Vd, s.n + dt * (b1 * a1.n + b2 * a2.n + b3 * a3.n),
                         s.h + dt * (b1 * a1.h + b2 * a2.h + b3 * a3.h), s.l + dt * (b1 * a1.l + b2 * a2.l + b3 * a3.l),
                         s.r + dt * (b1 * a1.r + b2 * a2.r + b3 * a3.r), s.c + dt * (b1 * a1.c + b2 * a2.c + b3 * a3.c),
                         s.Ca + dt * (b1 * a1.Ca + b2 * a2.Ca + b3 * a3.Ca), s.time + dt);

    const double q2 = 0.005430430675258792, q4 = 0.1720970973419255;
    s.Vs = s.Vs + dt * (a1.Vs / 6 - q2 * a2.Vs + 2 * a3.Vs / 3 + q4 * a4.Vs) + sq * p.sigma_s * J1s * 100000 / (RA_As * RA_cm);
    s.Vd = s.Vd + dt * (a1.Vd / 6 - q2 * a2.Vd + 2 * a3.Vd / 3 + q4 * a4.Vd) + sq * p.sigma_d * J1d * 100000 / (RA_Ad * RA_cm);
    s.Ca = s.Ca + dt * (a1.Ca / 6 - q2 * a2.Ca + 2 * a3.Ca / 3 + q4 * a4.Ca);
    s.n = s.n + dt * (a1.n / 6 - q2 * a2.n + 2 * a3.n / 3 + q4 * a4.n);
    s.l = s.l + dt * (a1.l / 6 - q2 * a2.l + 2 * a3.l / 3 + q4 * a4.l);
    s.h = s.h + dt * (a1.h / 6 - q2 * a2.h + 2 * a3.h / 3 + q4 * a4.h);
    s.r = s.r + dt * (a1.r / 6 - q2 * a2.r + 2 * a3.r / 3 + q4 * a4.r);
    s.c = s.c + dt * (a1.c / 6 - q2 * a2.c + 2 * a3.c / 3 + q4 * a4.c);

    double t1 = s.time + dt;
    s.Gexc_d = s.Gexc_d * std::exp(-(t1 - s.time) / RA_tExc);
    s.Gexc_s = s.Gexc_s * std::exp(-(t1 - s.time) / RA_tExc);
    s.Ginh_d = s.Ginh_d * std::exp(-(t1 - s.time) / RA_tInh);
    s.Ginh_s = s.Ginh_s * std::exp(-(t1 - s.time) / RA_tInh);
    s.time = s.time + dt;
}

/* Debraband_step_no_target_update, HH2_test.cpp:535-545: check then step.  The
 * four indices are drawn in the order ind1s, ind2s, ind1d, ind2d
 * (HH2_test.cpp:640-643). */
void ra_step(RAState& s, const RAParams& p, ugo_stream& noise)
{
    ra_state_check(s);
    int i1s = ugo_point_index(ugo_stream_word(&noise));
    int i2s = ugo_point_index(ugo_stream_word(&noise));
    int i1d = ugo_point_index(ugo_stream_word(&noise));
    int i2d = ugo_point_index(ugo_stream_word(&noise));
    ra_debrabant(s, p, ra_point_value(i1s), ra_point_value(i2s), ra_point_value(i1d), ra_point_value(i2d));
}

bool ra_bad_values(const RAState& s)
{
    /* check_bad_values, HH2_test.cpp:244-260 */
    if ((s.Vs > 100) || (s.Vs < -200)) return true;
    if (std::isnan(s.Vs)) return true;
    if ((s.Vd > 100) || (s.Vd < -200)) return true;
    if (std::isnan(s.Vd)) return true;
    return false;
}

/* ------------------------------------------------------------------------ */
/* HVC(I) interneuron: c++/src/HHI_buffer.cpp, c++/include/HHI_buffer.h        */
/* ------------------------------------------------------------------------ */

/* HHI_buffer.cpp:13-37 */
const double I_cm = 1.0, I_A = 6000;
const double I_Ena = 55.0, I_Ek = -80.0, I_El = -65.0, I_Ei = -75.0;
const double I_gNa = 100.0, I_gKdr = 20.0, I_gKHT = 500.0, I_gL = 0.1;
const double I_tExc = 2.0, I_tInh = 5.0;
const double I_threshold = -20.0, I_spike_margin = 5.0;
const double I_G_noise = 0.45, I_lambda = 250.0;

struct IState {
    double V, n, m, h, w, Gexc, Ginh, time;
    double noise_exc, noise_inh;
    int flag, Nspikes;
    bool fired;
};

/* rate functions, HHI_buffer.h:173-180 */
inline double i_an(double v) { return 0.15 * (v + 15) / (1 - std::exp(-(v + 15) / 10)); }
inline double i_bn(double v) { return 0.2 * std::exp(-(v + 25) / 80); }
inline double i_am(double v) { return (v + 22) / (1 - std::exp(-(v + 22) / 10)); }
inline double i_bm(double v) { return 40 * std::exp(-(v + 47) / 18); }
inline double i_ah(double v) { return 0.7 * std::exp(-(v + 34) / 20); }
inline double i_bh(double v) { return 10 / (1 + std::exp(-(v + 4) / 10)); }
inline double i_wInf(double v) { return 1 / (1 + std::exp(-v / 5)); }

/* draws the first noisy-spike time, HHI_buffer.cpp:217-239 */
double i_initial_noise_time(ugo_stream& st, double dt)
{
    double t = 1000 * (-std::log(1 - ugo_u01(ugo_stream_word(&st))) / I_lambda);
    while (t < dt) t = 1000 * (-std::log(1 - ugo_u01(ugo_stream_word(&st))) / I_lambda);
    return t;
}

/* set_to_rest, HHI_buffer.cpp:178-200 (Poisson noise is on for every HVC(I)). */
void i_set_to_rest(IState& s, ugo_stream& st, double dt)
{
    s.time = 0.0;
    s.V = -66; s.n = 0.125; s.m = 0.0; s.h = 0.99; s.w = 0.0;
    s.Gexc = 0.0; s.Ginh = 0.0;
    s.flag = 0; s.Nspikes = 0; s.fired = false;
    s.noise_exc = i_initial_noise_time(st, dt);
    s.noise_inh = i_initial_noise_time(st, dt);
}

/* HHI_buffer.cpp:260-276 */
void i_state_check(IState& s)
{
    if ((s.flag == 1) && (s.V < I_threshold - I_spike_margin)) {
        s.flag = 0;
        s.Nspikes++;
        s.fired = true;
    } else {
        s.fired = false;
        if ((s.flag == 0) && (s.V > I_threshold)) s.flag = 1;
    }
}

/* HHI_buffer.cpp:278-294 */
void i_noise_check(double time, double dt, double& G, double& noise_time, ugo_stream& st)
{
    if (time > noise_time) {
        G += ugo_random_G(I_G_noise, ugo_stream_word(&st));
        double rnd = 1000 * (-std::log(1 - ugo_u01(ugo_stream_word(&st))) / I_lambda);
        while (rnd < dt) {
            rnd = 1000 * (-std::log(1 - ugo_u01(ugo_stream_word(&st))) / I_lambda);
            G += ugo_random_G(I_G_noise, ugo_stream_word(&st));
        }
        noise_time = noise_time + rnd;
    }
}

struct IDerivs { double V, n, m, h, w; };

inline IDerivs i_rhs(const IState& s, double v, double t, double h, double w, double m3, double n4, double n, double m)
{
    /* HHI_buffer.cpp:739-747 */
    IDerivs k;
    double Ge = s.Gexc * std::exp(-(t - s.time) / I_tExc);
    double Gi = s.Ginh * std::exp(-(t - s.time) / I_tInh);
    const double I = 0.0;
    k.V = (-I_gL * (v - I_El) - I_gNa * h * m3 * (v - I_Ena) - I_gKdr * n4 * (v - I_Ek)
           - I_gKHT * w * (v - I_Ek) - Ge * v - Gi * (v - I_Ei) + 100000 * I / I_A) / I_cm;
    k.n = i_an(v) * (1 - n) - i_bn(v) * n;
    k.m = i_am(v) * (1 - m) - i_bm(v) * m;
    k.h = i_ah(v) * (1 - h) - i_bh(v) * h;
    k.w = (i_wInf(v) - w) / 1;
    return k;
}

/* Dormand-Prince 8 tableau as the reference writes it (HHI_buffer.cpp:426-690):
 * stages 2..6 take x + dt*(sum of small-integer multiples of k)/den,
 * stages 7..12 and the update take x + dt*(sum of num*k/den). */
struct DPTerm { int stage; double num; double den; };

const int DP_A_COUNT[5] = { 1, 2, 2, 3, 3 };
const int DP_A_STAGE[5][3] = { {0}, {0, 1}, {0, 2}, {0, 2, 3}, {0, 3, 4} };
const double DP_A_COEF[5][3] = { {1}, {1, 3}, {1, 3}, {20, -75, 75}, {3, 15, 12} };
const double DP_A_DEN[5] = { 18, 48, 32, 64, 80 };

const DPTerm DP_B7[] = { {0, 29443841, 614563906}, {3, 77736538, 692538347}, {4, -28693883, 1125000000},
                         {5, 23124283, 1800000000} };
const DPTerm DP_B8[] = { {0, 16016141, 946692911}, {3, 61564180, 158732637}, {4, 22789713, 633445777},
                         {5, 545815736, 2771057229.0}, {6, -180193667, 1043307555} };
const DPTerm DP_B9[] = { {0, 39632708, 573591083}, {3, -433636366, 683701615}, {4, -421739975, 2616292301.0},
                         {5, 100302831, 723423059}, {6, 790204164, 839813087}, {7, 800635310, 3783071287.0} };
const DPTerm DP_B10[] = { {0, 246121993, 1340847787}, {3, -37695042795.0, 15268766246.0}, {4, -309121744, 1061227803},
                          {5, -12992083, 490766935}, {6, 6005943493.0, 2108947869}, {7, 393006217, 1396673457},
                          {8, 123872331, 1001029789} };
const DPTerm DP_B11[] = { {0, -1028468189, 846180014}, {3, 8478235783.0, 508512852}, {4, 1311729495, 1432422823},
                          {5, -10304129995.0, 1701304382}, {6, -48777925059.0, 3047939560.0},
                          {7, 15336726248.0, 1032824649}, {8, -45442868181.0, 3398467696.0},
                          {9, 3065993473.0, 597172653} };
const DPTerm DP_B12[] = { {0, 185892177, 718116043}, {3, -3185094517.0, 667107341}, {4, -477755414, 1098053517},
                          {5, -703635378, 230739211}, {6, 5731566787.0, 1027545527}, {7, 5232866602.0, 850066563},
                          {8, -4093664535.0, 808688257}, {9, 3962137247.0, 1805957418}, {10, 65686358, 487910083} };
const DPTerm DP_OUT[] = { {0, 13451932, 455176623}, {5, -808719846, 976000145}, {6, 1757004468, 5645159321.0},
                          {7, 656045339, 265891186}, {8, -3867574721.0, 1518517206}, {9, 465885868, 322736535},
                          {10, 53011238, 667516719}, {11, 2, 45} };
/* stage times as (num * dt) / den */
const double DP_C_NUM[12] = { 0, 1, 1, 1, 5, 3, 59, 93, 5490023248.0, 13, 1201146811, 1 };
const double DP_C_DEN[12] = { 1, 18, 12, 8, 16, 8, 400, 200, 9719169821.0, 20, 12990119798.0, 1 };

inline double dp_sum_b(const DPTerm* terms, int count, const double* k)
{
    double acc = terms[0].num * k[terms[0].stage] / terms[0].den;
    for (int j = 1; j < count; ++j) acc = acc + terms[j].num * k[terms[j].stage] / terms[j].den;
    return acc;
}

/* One 12-stage DP8 step of (V, n, m, h, w), HHI_buffer.cpp:426-690. */
void i_dp8(IState& s, double dt)
{
    double kV[12], kn[12], km[12], kh[12], kw[12];
    const DPTerm* tabB[6] = { DP_B7, DP_B8, DP_B9, DP_B10, DP_B11, DP_B12 };
    const int cntB[6] = { 4, 5, 6, 7, 8, 9 };
    for (int st = 0; st < 12; ++st) {
        double v, n1, m1, h1, w1, t;
        if (st == 0) {
            v = s.V; n1 = s.n; m1 = s.m; h1 = s.h; w1 = s.w; t = s.time;
        } else if (st <= 5) {
            const int a = st - 1;
            double sV = 0, sn = 0, sm = 0, sh = 0, sw = 0;
            for (int j = 0; j < DP_A_COUNT[a]; ++j) {
                int q = DP_A_STAGE[a][j];
                double c = DP_A_COEF[a][j];
                if (j == 0) {
                    sV = c * kV[q]; sn = c * kn[q]; sm = c * km[q]; sh = c * kh[q]; sw = c * kw[q];
                } else {
                    sV = sV + c * kV[q]; sn = sn + c * kn[q]; sm = sm + c * km[q]; sh = sh + c * kh[q]; sw = sw + c * kw[q];
                }
            }
            m1 = s.m + dt * sm / DP_A_DEN[a];
            n1 = s.n + dt * sn / DP_A_DEN[a];
            h1 = s.h + dt * sh / DP_A_DEN[a];
            w1 = s.w + dt * sw / DP_A_DEN[a];
            v = s.V + dt * sV / DP_A_DEN[a];
            t = s.time + DP_C_NUM[st] * dt / DP_C_DEN[st];
        } else {
            const DPTerm* tb = tabB[st - 6];
            const int cnt = cntB[st - 6];
            m1 = s.m + dt * dp_sum_b(tb, cnt, km);
            n1 = s.n + dt * dp_sum_b(tb, cnt, kn);
            h1 = s.h + dt * dp_sum_b(tb, cnt, kh);
            w1 = s.w + dt * dp_sum_b(tb, cnt, kw);
            v = s.V + dt * dp_sum_b(tb, cnt, kV);
            t = (st == 11) ? s.time + dt : s.time + DP_C_NUM[st] * dt / DP_C_DEN[st];
        }
        double n4 = n1 * n1 * n1 * n1;
        double m3 = m1 * m1 * m1;
        IDerivs k = i_rhs(s, v, t, h1, w1, m3, n4, n1, m1);
        kV[st] = k.V; kn[st] = k.n; km[st] = k.m; kh[st] = k.h; kw[st] = k.w;
    }
    s.V = s.V + dt * dp_sum_b(DP_OUT, 8, kV);
    s.n = s.n + dt * dp_sum_b(DP_OUT, 8, kn);
    s.m = s.m + dt * dp_sum_b(DP_OUT, 8, km);
    s.h = s.h + dt * dp_sum_b(DP_OUT, 8, kh);
    s.w = s.w + dt * dp_sum_b(DP_OUT, 8, kw);
    double t1 = s.time + dt;
    s.Gexc = s.Gexc * std::exp(-(t1 - s.time) / I_tExc);
    s.Ginh = s.Ginh * std::exp(-(t1 - s.time) / I_tInh);
    s.time = s.time + dt;
}

/* DP8_step_no_target_update, HHI_buffer.cpp:332-339 with state_noise_check
 * (HHI_buffer.cpp:248-258): check, exc noise, inh noise, step. */
void i_step(IState& s, double dt, ugo_stream& st)
{
    i_state_check(s);
    i_noise_check(s.time, dt, s.Gexc, s.noise_exc, st);
    i_noise_check(s.time, dt, s.Ginh, s.noise_inh, st);
    i_dp8(s, dt);
}

/* ------------------------------------------------------------------------ */
/* Network constants, NetworkGrowthSimulator.cpp:13-26                          */
/* ------------------------------------------------------------------------ */
const double STDP_WINDOW = 100.0;
const double WAITING_TIME = 100.0;
const double TIMESTEP = 0.02;
const double NETWORK_UPDATE_FREQUENCY = 0.25;
const double TRIAL_DURATION = 500.0;
const double EXPERIMENTAL_INTERNEURON_DISTANCE = 40.0;
const double MIN_INTERSOMATIC_DISTANCE = 10.0;
const double G_TRAINING_KICK = 3.0;
const double MATURATION_SCALE_SPONTANEOUS = 100000;
const double MATURATION_SCALE_DRIVEN = 1000;
const double EXPERIMENTAL_AXONAL_DELAY_PER_MICRON = 0.01;
const double EVENT_WINDOW = 30.0;      /* NetworkGrowthSimulator.cpp:8841 */
const int ROBUSTNESS_WINDOW = 1000;    /* NetworkGrowthSimulator.cpp:9586 */
const double DRIVEN_THRESHOLD = 0.50;  /* NetworkGrowthSimulator.cpp:9588 */

double distance_on_sphere(double x1, double y1, double z1, double x2, double y2, double z2)
{
    double tmp = x1 * x2 + y1 * y2 + z1 * z2;
    if (tmp > 1.0) return 0.0;
    return std::acos(tmp);
}

typedef std::pair<double, int> Event;

/* upper_bound insertion into a (time, target)-sorted queue
 * (NetworkGrowthSimulator.cpp:8977-8985). */
void queue_insert(std::vector<Event>& q, double t, int target)
{
    Event e(t, target);
    auto it = std::upper_bound(q.begin(), q.end(), e);
    q.insert(it, e);
}

struct Conn {
    std::vector<int> tgt;
    std::vector<double> w, d, len;
};

} // namespace

struct ugo_net {
    int n_ra, n_i;
    int num_steps;
    uint64_t seed;
    uint32_t net_id;
    ugo_synaptic_params syn;
    ugo_maturation_params mat;
    ugo_noise_params noise;
    ugo_connection_params conn;

    std::vector<RAState> ra;
    std::vector<IState> in;
    std::vector<Conn> ra2i, i2ra;
    std::vector<double> W, D, L;                 /* dense RA->RA */
    std::vector<unsigned char> active, super;    /* dense indicators */
    std::vector<std::vector<int>> active_list, super_list;
    std::vector<int> remodeled, mature, trials_after_replacement;
    std::vector<double> rest_potential, gca, maturation_scale, firing_rate_long;
    std::vector<std::vector<int>> hist;          /* activity history, newest first */
    std::vector<int> training;                   /* sorted training ids */
    std::vector<double> spread;                  /* spread time per RA (0 for non-training) */
    std::vector<double> ra_xyz, i_xyz;

    double mean_injection_time;
    std::vector<double> T;                        /* internal_time after step t */
    std::vector<int> spk_soma_n, spk_soma_s, spk_dend_n, spk_dend_s, spk_i_n, spk_i_s;
    std::vector<int> replaced;

    std::vector<int> trace_ra, trace_i;
    std::vector<double> trace_ra_buf, trace_i_buf;
    double ginh_res;                              /* inhibition tracking resolution (0: off) */
    std::vector<double> ginh;                     /* [n_ra][points] Ginh_d record (Ginh_global) */
    bool log_deliveries;
    std::vector<int> delivery_log;

    std::vector<ugo_stream> ra_noise, i_noise;

    /* Step gate of a trial run on a worker thread (ugo_trial_begin / _advance / _end):
     * the trial waits before step t until t < gate_until. */
    std::mutex gate_mu;
    std::condition_variable gate_cv;
    bool gated = false;
    int gate_until = INT_MAX;
    int gate_at = 0;          /* the step the trial waits at; num_steps once it has finished */
    bool gate_done = false;
    int gate_rc = 0;
    std::thread gate_worker;
};

namespace {

RAParams ra_params(const ugo_net* net, int i)
{
    RAParams p;
    p.EL = net->rest_potential[i];
    p.GdCa = net->gca[i];
    p.mu_s = net->noise.white_noise_mean_soma;
    p.sigma_s = net->noise.white_noise_std_soma;
    p.mu_d = net->noise.white_noise_mean_dend;
    p.sigma_d = net->noise.white_noise_std_dend;
    p.dt = TIMESTEP;
    return p;
}

/* update_synapse, NetworkGrowthSimulator.cpp:16546-16592 */
void update_synapse(ugo_net* net, int i, int j)
{
    const int N = net->n_ra;
    const double w = net->W[(size_t)i * N + j];
    unsigned char& act = net->active[(size_t)i * N + j];
    unsigned char& sup = net->super[(size_t)i * N + j];
    const ugo_synaptic_params& sp = net->syn;
    if ((w >= sp.ACTIVATION_THRESHOLD) && (act == 0) && (net->remodeled[i] == 0)) {
        act = 1;
        net->active_list[i].push_back(j);
    }
    if ((w >= sp.SUPERSYNAPSE_THRESHOLD) && (sup == 0) && ((int)net->super_list[i].size() < sp.Nss)) {
        sup = 1;
        net->super_list[i].push_back(j);
    }
    if ((w < sp.SUPERSYNAPSE_THRESHOLD) && (sup == 1)) {
        sup = 0;
        net->remodeled[i] = 0;
        auto pos = std::find(net->super_list[i].begin(), net->super_list[i].end(), j);
        if (pos != net->super_list[i].end()) net->super_list[i].erase(pos);
    }
    if ((w < sp.ACTIVATION_THRESHOLD) && (act == 1)) {
        act = 0;
        auto pos = std::find(net->active_list[i].begin(), net->active_list[i].end(), j);
        if (pos != net->active_list[i].end()) net->active_list[i].erase(pos);
    }
}

/* LTP, NetworkGrowthSimulator.cpp:16615-16634 */
void LTP(const ugo_synaptic_params& sp, double& w, double dt)
{
    if (dt <= sp.T_0) return;
    if (dt <= sp.T_0 + sp.T_P)
        w = w + sp.A_P * (dt - sp.T_0) / sp.T_P;
    else
        w = w + sp.A_P * std::exp(-(dt - sp.T_0 - sp.T_P) / sp.TAU_P);
    if (w > sp.WEIGHT_MAX) w = sp.WEIGHT_MAX;
    if (w < 0) w = 0;
}

/* LTD, NetworkGrowthSimulator.cpp:16636-16652 */
void LTD(const ugo_synaptic_params& sp, double& w, double dt)
{
    if (dt > sp.T_0) return;
    if (dt >= sp.T_0 - sp.T_D)
        w = w + w * sp.A_D * (dt - sp.T_0) / sp.T_D;
    else
        w = w - w * sp.A_D * std::exp((dt - sp.T_0 + sp.T_D) / sp.TAU_D);
    if (w < 0) w = 0;
}

/* axon_remodeling, NetworkGrowthSimulator.cpp:16363-16415 */
void axon_remodeling(ugo_net* net, int i)
{
    const int N = net->n_ra;
    for (size_t k = 0; k < net->active_list[i].size(); ++k) net->active[(size_t)i * N + net->active_list[i][k]] = 0;
    for (size_t k = 0; k < net->super_list[i].size(); ++k) net->active[(size_t)i * N + net->super_list[i][k]] = 1;
    net->active_list[i] = net->super_list[i];
    net->remodeled[i] = 1;
}

void build_time_table(ugo_net* net)
{
    net->T.assign(net->num_steps, 0.0);
    double t = 0;
    for (int s = 1; s < net->num_steps; ++s) {
        t += TIMESTEP;
        net->T[s] = t;
    }
}

void record_traces(ugo_net* net)
{
    for (int k = 0; k < (int)net->trace_ra.size(); ++k) {
        const RAState& s = net->ra[net->trace_ra[k]];
        double row[10] = { s.Vs, s.Vd, s.n, s.h, s.l, s.r, s.c, s.Ca, s.Gexc_d, s.Ginh_d };
        net->trace_ra_buf.insert(net->trace_ra_buf.end(), row, row + 10);
    }
    for (int k = 0; k < (int)net->trace_i.size(); ++k) {
        const IState& s = net->in[net->trace_i[k]];
        double row[7] = { s.V, s.n, s.m, s.h, s.w, s.Gexc, s.Ginh };
        net->trace_i_buf.insert(net->trace_i_buf.end(), row, row + 7);
    }
}

void init_trial_noise(ugo_net* net, uint32_t trial)
{
    net->ra_noise.resize(net->n_ra);
    net->i_noise.resize(net->n_i);
    for (int i = 0; i < net->n_ra; ++i)
        ugo_stream_init(&net->ra_noise[i], net->seed, UGO_KIND_RA_WHITE, net->net_id, (uint32_t)i, trial);
    for (int i = 0; i < net->n_i; ++i) {
        ugo_stream_init(&net->i_noise[i], net->seed, UGO_KIND_I_POISSON, net->net_id, (uint32_t)i, trial);
        /* every trial starts from set_to_rest, which redraws the noise times */
        i_set_to_rest(net->in[i], net->i_noise[i], TIMESTEP);
    }
    for (int i = 0; i < net->n_ra; ++i) ra_set_to_rest(net->ra[i]);
}

/* One trial; growth == false is trial_no_stdp_fixedSpread
 * (NetworkGrowthSimulator.cpp:12747-13117), growth == true is
 * trial_1stSoma_pre_1stSoma_post_delays_fixedSpread (:8839-9571). */
int run_trial(ugo_net* net, bool growth, bool training, uint32_t trial)
{
    const int NRA = net->n_ra, NI = net->n_i;
    const ugo_synaptic_params& sp = net->syn;
    build_time_table(net);
    init_trial_noise(net, trial);

    net->spk_soma_n.clear(); net->spk_soma_s.clear();
    net->spk_dend_n.clear(); net->spk_dend_s.clear();
    net->spk_i_n.clear(); net->spk_i_s.clear();
    net->trace_ra_buf.clear(); net->trace_i_buf.clear();
    net->delivery_log.clear();

    std::vector<double> upd_Ge_RA(NRA, 0.0), upd_Gi_RA(NRA, 0.0), upd_Ge_I(NI, 0.0);
    std::vector<std::vector<Event>> q_rara(NRA), q_rai(NRA), q_ira(NI);
    std::vector<std::vector<std::vector<double>>> pre_events;   /* growth only */
    std::vector<std::vector<double>> post_events(NRA);
    std::vector<int> new_post;
    std::vector<char> injected(NRA, 0);
    std::vector<char> is_training(NRA, 0);
    for (int id : net->training) is_training[id] = 1;
    if (growth) {
        pre_events.resize(NRA);
        for (int i = 0; i < NRA; ++i) pre_events[i].resize(NRA);
    }

    if (growth) {
        ugo_stream ts;
        ugo_stream_init(&ts, net->seed, UGO_KIND_TRIAL, net->net_id, 0, trial);
        net->mean_injection_time = WAITING_TIME + ugo_random_G(TRIAL_DURATION - 2 * WAITING_TIME, ugo_stream_word(&ts));
    } else {
        net->mean_injection_time = 100;
    }
    const bool kick_on = growth ? training : true;

    double internal_time = 0;
    double network_time = NETWORK_UPDATE_FREQUENCY;
    int flag_ra_inh = 0, flag_ra_exc = 0, flag_i_exc = 0, flag_post = 0;
    const int num_steps = net->num_steps;

    if (!net->trace_ra.empty() || !net->trace_i.empty()) record_traces(net);
    /* inhibition tracking (:8158-8160): Ginh_d at the trial's start, then at the first step
     * at or after each multiple of the resolution (:8432-8442) */
    const int ginh_points = net->ginh_res > 0 ? (int)(num_steps * TIMESTEP / net->ginh_res) : 0;
    int ginh_pos = 1;
    if (ginh_points > 0) {
        if (net->ginh.size() != (size_t)NRA * ginh_points) net->ginh.assign((size_t)NRA * ginh_points, 0.0);
        for (int i = 0; i < NRA; ++i) net->ginh[(size_t)i * ginh_points] = net->ra[i].Ginh_d;
    }

    for (int t = 1; t < num_steps; ++t) {
        if (net->gated) {
            std::unique_lock<std::mutex> lk(net->gate_mu);
            net->gate_at = t;
            net->gate_cv.notify_all();
            net->gate_cv.wait(lk, [&] { return t < net->gate_until; });
        }
        internal_time += TIMESTEP;
        for (int i = 0; i < NRA; ++i) {
            RAState& s = net->ra[i];
            if (kick_on && is_training[i] && !injected[i]) {
                if (internal_time > net->spread[i] + net->mean_injection_time) {
                    s.Gexc_d += G_TRAINING_KICK;   /* raiseE, HH2_test.cpp:439-442 */
                    injected[i] = 1;
                }
            }
            RAParams p = ra_params(net, i);
            ra_step(s, p, net->ra_noise[i]);

            if (s.fired_soma) {
                net->spk_soma_n.push_back(i);
                net->spk_soma_s.push_back(t);
                if (growth) {
                    if (post_events[i].empty()) {
                        new_post.push_back(i);
                        flag_post = 1;
                    } else if (internal_time > post_events[i].back() + EVENT_WINDOW) {
                        new_post.push_back(i);
                        flag_post = 1;
                    }
                }
                const Conn& ci = net->ra2i[i];
                for (size_t j = 0; j < ci.tgt.size(); ++j) queue_insert(q_rai[i], internal_time + ci.d[j], (int)j);
                if (growth) {
                    if ((int)net->super_list[i].size() == sp.Nss) {
                        for (size_t k = 0; k < net->super_list[i].size(); ++k) {
                            int tg = net->super_list[i][k];
                            queue_insert(q_rara[i], internal_time + net->D[(size_t)i * NRA + tg], tg);
                        }
                    } else {
                        for (int j = 0; j < NRA; ++j)
                            if (j != i) queue_insert(q_rara[i], internal_time + net->D[(size_t)i * NRA + j], j);
                    }
                } else {
                    for (size_t k = 0; k < net->active_list[i].size(); ++k) {
                        int tg = net->active_list[i][k];
                        queue_insert(q_rara[i], internal_time + net->D[(size_t)i * NRA + tg], tg);
                    }
                }
            }

            /* RA -> I drain (:9039-9062) */
            {
                auto& q = q_rai[i];
                size_t k = 0;
                for (; k < q.size(); ++k) {
                    if (internal_time >= q[k].first) {
                        flag_i_exc = 1;
                        int pos = q[k].second;
                        upd_Ge_I[net->ra2i[i].tgt[pos]] += net->ra2i[i].w[pos];
                    } else break;
                }
                q.erase(q.begin(), q.begin() + k);
            }
            /* RA -> RA drain (:9069-9191; test trial :12887-12938) */
            {
                auto& q = q_rara[i];
                size_t k = 0;
                for (; k < q.size(); ++k) {
                    double delivery_time = q[k].first;
                    if (!(internal_time >= delivery_time)) break;
                    int tg = q[k].second;
                    if (net->log_deliveries) {
                        net->delivery_log.push_back(i);
                        net->delivery_log.push_back(tg);
                        net->delivery_log.push_back(t);
                    }
                    size_t ij = (size_t)i * NRA + tg;
                    if (!growth) {
                        flag_ra_exc = 1;
                        upd_Ge_RA[tg] += net->W[ij];
                        continue;
                    }
                    if (net->active[ij] == 1) {
                        flag_ra_exc = 1;
                        upd_Ge_RA[tg] += net->W[ij];
                    }
                    bool new_pre = false;
                    std::vector<double>& pe = pre_events[i][tg];
                    if (!pe.empty()) {
                        if (delivery_time > pe.back() + EVENT_WINDOW) {
                            pe.push_back(delivery_time);
                            new_pre = true;
                        }
                    } else {
                        pe.push_back(delivery_time);
                        new_pre = true;
                    }
                    if (!new_pre) continue;
                    if ((int)net->super_list[i].size() == sp.Nss) {
                        if (net->super[ij] == 1) {
                            const std::vector<double>& po = post_events[tg];
                            if (!po.empty()) {
                                auto it0 = std::lower_bound(po.begin(), po.end(), internal_time - STDP_WINDOW);
                                for (auto it = it0; it != po.end(); ++it) {
                                    double dt = *it - delivery_time;
                                    LTD(sp, net->W[ij], dt);
                                    update_synapse(net, i, tg);
                                }
                            }
                        }
                        if ((int)net->super_list[i].size() < sp.Nss)
                            for (int j = 0; j < NRA; ++j) update_synapse(net, i, j);
                    } else {
                        const std::vector<double>& po = post_events[tg];
                        if (!po.empty()) {
                            auto it0 = std::lower_bound(po.begin(), po.end(), internal_time - STDP_WINDOW);
                            for (auto it = it0; it != po.end(); ++it) {
                                double dt = *it - delivery_time;
                                LTD(sp, net->W[ij], dt);
                                update_synapse(net, i, tg);
                            }
                        }
                    }
                }
                q.erase(q.begin(), q.begin() + k);
            }
            if (s.fired_dend) {
                net->spk_dend_n.push_back(i);
                net->spk_dend_s.push_back(t);
            }
        }
        if (ginh_points > 0 && internal_time >= static_cast<double>(ginh_pos) * net->ginh_res) {
            if (ginh_pos < ginh_points)
                for (int i = 0; i < NRA; ++i) net->ginh[(size_t)i * ginh_points + ginh_pos] = net->ra[i].Ginh_d;
            ginh_pos += 1;
        }

        for (int i = 0; i < NI; ++i) {
            IState& s = net->in[i];
            i_step(s, TIMESTEP, net->i_noise[i]);
            if (s.fired) {
                net->spk_i_n.push_back(i);
                net->spk_i_s.push_back(t);
                const Conn& ci = net->i2ra[i];
                for (size_t j = 0; j < ci.tgt.size(); ++j) queue_insert(q_ira[i], internal_time + ci.d[j], (int)j);
            }
            auto& q = q_ira[i];
            size_t k = 0;
            for (; k < q.size(); ++k) {
                if (internal_time >= q[k].first) {
                    flag_ra_inh = 1;
                    int pos = q[k].second;
                    upd_Gi_RA[net->i2ra[i].tgt[pos]] += net->i2ra[i].w[pos];
                } else break;
            }
            q.erase(q.begin(), q.begin() + k);
        }

        /* network synchronization (:9291-9564; test trial :13036-13115) */
        if ((internal_time > network_time) || (t == num_steps - 1)) {
            if (flag_ra_inh > 0) {
                for (int i = 0; i < NRA; ++i) net->ra[i].Ginh_d += upd_Gi_RA[i];       /* raiseI */
                flag_ra_inh = 0;
                std::fill(upd_Gi_RA.begin(), upd_Gi_RA.end(), 0.0);
            }
            if (flag_i_exc > 0) {
                for (int i = 0; i < NI; ++i) net->in[i].Gexc += upd_Ge_I[i];            /* raiseE */
                flag_i_exc = 0;
                std::fill(upd_Ge_I.begin(), upd_Ge_I.end(), 0.0);
            }
            if (flag_ra_exc > 0) {
                for (int i = 0; i < NRA; ++i) net->ra[i].Gexc_d += upd_Ge_RA[i] / RA_Ad;  /* raiseExcWeight */
                flag_ra_exc = 0;
                std::fill(upd_Ge_RA.begin(), upd_Ge_RA.end(), 0.0);
            }
            if (growth && flag_post > 0) {
                flag_post = 0;
                for (size_t k = 0; k < new_post.size(); ++k) post_events[new_post[k]].push_back(internal_time);
                for (int i = 0; i < NRA; ++i) {
                    const bool saturated = (int)net->super_list[i].size() == sp.Nss;
                    for (size_t k = 0; k < new_post.size(); ++k) {
                        int post = new_post[k];
                        if (post == i) continue;
                        if (saturated) {
                            auto pos = std::find(net->super_list[i].begin(), net->super_list[i].end(), post);
                            if (pos == net->super_list[i].end()) continue;
                        }
                        std::vector<double>& pe = pre_events[i][post];
                        if (pe.empty()) continue;
                        auto it0 = std::lower_bound(pe.begin(), pe.end(), internal_time - STDP_WINDOW);
                        for (auto it = it0; it != pe.end(); ++it) {
                            double dt = internal_time - *it;
                            double& w = net->W[(size_t)i * NRA + post];
                            if (dt <= sp.T_0) LTD(sp, w, dt);
                            else LTP(sp, w, dt);
                            update_synapse(net, i, post);
                        }
                    }
                }
                for (int i = 0; i < NRA; ++i)
                    if (((int)net->super_list[i].size() == sp.Nss) && (net->remodeled[i] == 0)) axon_remodeling(net, i);
                new_post.clear();
            }
            network_time += NETWORK_UPDATE_FREQUENCY;
        }
        if (!net->trace_ra.empty() || !net->trace_i.empty()) record_traces(net);
    }

    if (growth) {
        /* potentiation_decay (:16346-16361) then update_all_synapses (:16432-16443) */
        for (int i = 0; i < NRA; ++i)
            for (int j = 0; j < NRA; ++j) {
                double& w = net->W[(size_t)i * NRA + j];
                if (w >= sp.SUPERSYNAPSE_THRESHOLD) w -= sp.BETA_SUPERSYNAPSE;
                else w -= sp.BETA;
                if (w < 0) w = 0;
            }
        for (int i = 0; i < NRA; ++i)
            for (int j = 0; j < NRA; ++j) update_synapse(net, i, j);
    }
    for (int i = 0; i < NRA; ++i)
        if (ra_bad_values(net->ra[i])) return -1;
    return 0;
}

/* check_neuron_activity, NetworkGrowthSimulator.cpp:9573-9627 */
void check_neuron_activity(ugo_net* net, std::vector<int>& to_replace)
{
    const int W = net->mat.RATE_WINDOW_LONG;
    std::vector<int> count(net->n_ra, 0);
    for (size_t k = 0; k < net->spk_soma_n.size(); ++k) count[net->spk_soma_n[k]]++;
    for (int i = 0; i < net->n_ra; ++i) {
        std::vector<int>& h = net->hist[i];
        h.insert(h.begin(), count[i]);     /* push_front into a full circular buffer */
        h.pop_back();
        double sum = 0.0;
        for (int k = 0; k < W; ++k) sum += h[k];
        net->firing_rate_long[i] = sum / (double)W;
        double robust = 0.0;
        for (int k = 0; k < ROBUSTNESS_WINDOW; ++k)
            if (h[k] > 0) robust += 1;
        robust = robust / (double)ROBUSTNESS_WINDOW;
        if ((robust >= DRIVEN_THRESHOLD) && (net->maturation_scale[i] != MATURATION_SCALE_DRIVEN))
            net->maturation_scale[i] = MATURATION_SCALE_DRIVEN;
        if ((robust < net->mat.DEATH_RATE_THRESHOLD) && (net->trials_after_replacement[i] > ROBUSTNESS_WINDOW))
            to_replace.push_back(i);
    }
}

/* update_neuron_properties_sameDendrite_diffMaturationRate, :2152-2183 */
void update_maturation(ugo_net* net)
{
    const ugo_maturation_params& mp = net->mat;
    for (int i = 0; i < net->n_ra; ++i) {
        if (net->mature[i] != 1) {
            net->rest_potential[i] = net->rest_potential[i] + (net->rest_potential[i] - mp.E_REST_MATURE)
                                                              * (std::exp(-1.0 / net->maturation_scale[i]) - 1);
            net->gca[i] = net->gca[i] + (net->gca[i] - mp.GCA_MATURE) * (std::exp(-1.0 / net->maturation_scale[i]) - 1);
            if ((net->gca[i] >= mp.GCA_MATURE - 0.5) || (net->rest_potential[i] <= mp.E_REST_MATURE - 0.5)) {
                net->gca[i] = mp.GCA_MATURE;
                net->rest_potential[i] = mp.E_REST_MATURE;
                net->mature[i] = 1;
            }
        }
    }
}

double p_ra2i(const ugo_connection_params& c, double d)
{
    double sigma_square = c.SIGMA_RA2I * c.SIGMA_RA2I;
    return c.A_RA2I * std::exp(-d * d / (2 * sigma_square));
}

double p_i2ra(const ugo_connection_params& c, double d)
{
    double sigma_square = c.SIGMA_I2RA * c.SIGMA_I2RA;
    return c.B_I2RA * std::exp(-d * d / (2 * sigma_square));
}

/* replace_neurons, NetworkGrowthSimulator.cpp:15869-15881, with
 * remove_neurons_from_network (:15757-15859), sample_coordinates_for_replaced
 * (:157-220), sample_connectionsAndDelays_for_replaced (:528-618) and
 * update_replaced_neurons (:2109-2134). */
void replace_neurons(ugo_net* net, const std::vector<int>& rep, uint32_t trial)
{
    const int N = net->n_ra, NI = net->n_i;
    for (int i = 0; i < N; ++i) {
        for (size_t k = 0; k < rep.size(); ++k) {
            int j = rep[k];
            size_t ij = (size_t)i * N + j;
            if (net->active[ij] == 1) {
                auto it = std::find(net->active_list[i].begin(), net->active_list[i].end(), j);
                if (it != net->active_list[i].end()) net->active_list[i].erase(it);
                net->active[ij] = 0;
            }
            if (net->super[ij] == 1) {
                auto it = std::find(net->super_list[i].begin(), net->super_list[i].end(), j);
                if (it != net->super_list[i].end()) net->super_list[i].erase(it);
                net->super[ij] = 0;
                net->remodeled[i] = 0;
            }
            net->W[ij] = 0.0;
        }
    }
    for (size_t k = 0; k < rep.size(); ++k) {
        int r = rep[k];
        net->active_list[r].clear();
        net->super_list[r].clear();
        for (int j = 0; j < N; ++j) {
            net->super[(size_t)r * N + j] = 0;
            net->active[(size_t)r * N + j] = 0;
            net->W[(size_t)r * N + j] = 0.0;
        }
    }
    for (int i = 0; i < NI; ++i) {
        for (size_t k = 0; k < rep.size(); ++k) {
            Conn& c = net->i2ra[i];
            auto it = std::find(c.tgt.begin(), c.tgt.end(), rep[k]);
            if (it != c.tgt.end()) {
                size_t ind = (size_t)(it - c.tgt.begin());
                c.tgt.erase(it);
                c.w.erase(c.w.begin() + ind);
                c.len.erase(c.len.begin() + ind);
                c.d.erase(c.d.begin() + ind);
            }
        }
    }
    for (size_t k = 0; k < rep.size(); ++k) {
        Conn& c = net->ra2i[rep[k]];
        c.tgt.clear(); c.w.clear(); c.d.clear(); c.len.clear();
    }

    ugo_stream rs;
    ugo_stream_init(&rs, net->seed, UGO_KIND_REPLACE, net->net_id, 0, trial);
    const ugo_connection_params& cp = net->conn;
    const double model_dist = cp.model_interneuron_distance;
    const double pi = 3.14159265358979323846;
    const double too_close = model_dist * MIN_INTERSOMATIC_DISTANCE / EXPERIMENTAL_INTERNEURON_DISTANCE;

    std::vector<int> fixed;
    {
        std::vector<char> is_rep(N, 0);
        for (int r : rep) is_rep[r] = 1;
        for (int i = 0; i < N; ++i) if (!is_rep[i]) fixed.push_back(i);
    }
    double* X = net->ra_xyz.data();
    const double* XI = net->i_xyz.data();
    for (size_t k = 0; k < rep.size(); ++k) {
        double tx = 0, ty = 0, tz = 0;
        bool close = true;
        while (close) {
            close = false;
            double z = 2 * ugo_random_G(1.0, ugo_stream_word(&rs)) - 1;
            double phi = ugo_random_G(2.0 * pi, ugo_stream_word(&rs));
            tx = std::sin(std::acos(z)) * std::cos(phi);
            ty = std::sin(std::acos(z)) * std::sin(phi);
            tz = z;
            for (int j = 0; j < NI; ++j)
                if (distance_on_sphere(tx, ty, tz, XI[3 * j], XI[3 * j + 1], XI[3 * j + 2]) < too_close) { close = true; break; }
            if (!close)
                for (size_t f = 0; f < fixed.size(); ++f) {
                    int id = fixed[f];
                    if (distance_on_sphere(tx, ty, tz, X[3 * id], X[3 * id + 1], X[3 * id + 2]) < too_close) { close = true; break; }
                }
        }
        X[3 * rep[k]] = tx; X[3 * rep[k] + 1] = ty; X[3 * rep[k] + 2] = tz;
        fixed.push_back(rep[k]);
    }
    for (size_t k = 0; k < rep.size(); ++k) {
        int id = rep[k];
        for (int j = 0; j < NI; ++j) {
            double d = distance_on_sphere(X[3 * id], X[3 * id + 1], X[3 * id + 2], XI[3 * j], XI[3 * j + 1], XI[3 * j + 2])
                       * EXPERIMENTAL_INTERNEURON_DISTANCE / model_dist;
            if (ugo_random_G(1, ugo_stream_word(&rs)) < p_ra2i(cp, d)) {
                double G = ugo_random_G(1.0, ugo_stream_word(&rs)) * cp.Gei_max;
                Conn& c = net->ra2i[id];
                c.w.push_back(G); c.tgt.push_back(j); c.len.push_back(d);
                c.d.push_back(d * EXPERIMENTAL_AXONAL_DELAY_PER_MICRON * cp.delay_constant);
            }
        }
    }
    for (int i = 0; i < NI; ++i) {
        for (size_t k = 0; k < rep.size(); ++k) {
            int id = rep[k];
            double d = distance_on_sphere(XI[3 * i], XI[3 * i + 1], XI[3 * i + 2], X[3 * id], X[3 * id + 1], X[3 * id + 2])
                       * EXPERIMENTAL_INTERNEURON_DISTANCE / model_dist;
            if (ugo_random_G(1, ugo_stream_word(&rs)) < p_i2ra(cp, d)) {
                double G = ugo_random_G(1.0, ugo_stream_word(&rs)) * cp.Gie_max;
                Conn& c = net->i2ra[i];
                c.w.push_back(G); c.tgt.push_back(id); c.len.push_back(d);
                c.d.push_back(d * EXPERIMENTAL_AXONAL_DELAY_PER_MICRON * cp.delay_constant);
            }
        }
    }
    for (int i = 0; i < N; ++i)
        for (size_t k = 0; k < rep.size(); ++k) {
            int tg = rep[k];
            double len = (tg != i) ? distance_on_sphere(X[3 * i], X[3 * i + 1], X[3 * i + 2], X[3 * tg], X[3 * tg + 1], X[3 * tg + 2])
                                         * EXPERIMENTAL_INTERNEURON_DISTANCE / model_dist
                                   : 0.0;
            net->L[(size_t)i * N + tg] = len;
            net->D[(size_t)i * N + tg] = len * EXPERIMENTAL_AXONAL_DELAY_PER_MICRON * cp.delay_constant;
        }
    for (size_t k = 0; k < rep.size(); ++k)
        for (int j = 0; j < N; ++j) {
            int src = rep[k];
            double len = (j != src) ? distance_on_sphere(X[3 * src], X[3 * src + 1], X[3 * src + 2], X[3 * j], X[3 * j + 1], X[3 * j + 2])
                                          * EXPERIMENTAL_INTERNEURON_DISTANCE / model_dist
                                    : 0.0;
            net->L[(size_t)src * N + j] = len;
            net->D[(size_t)src * N + j] = len * EXPERIMENTAL_AXONAL_DELAY_PER_MICRON * cp.delay_constant;
        }
    for (size_t k = 0; k < rep.size(); ++k) {
        int r = rep[k];
        net->rest_potential[r] = net->mat.E_REST_IMMATURE;
        net->gca[r] = net->mat.GCA_IMMATURE;
        net->mature[r] = 0;
        net->maturation_scale[r] = MATURATION_SCALE_SPONTANEOUS;
        net->remodeled[r] = 0;
        net->trials_after_replacement[r] = 0;
        std::fill(net->hist[r].begin(), net->hist[r].end(), 0);
    }
}

void set_csr(std::vector<Conn>& dst, int n_src, const int32_t* off, const int32_t* tgt, const double* w,
             const double* d, const double* len)
{
    dst.assign(n_src, Conn());
    for (int i = 0; i < n_src; ++i)
        for (int k = off[i]; k < off[i + 1]; ++k) {
            dst[i].tgt.push_back(tgt[k]);
            dst[i].w.push_back(w[k]);
            dst[i].d.push_back(d[k]);
            dst[i].len.push_back(len ? len[k] : 0.0);
        }
}

} // namespace

extern "C" {

ugo_net* ugo_new(int32_t n_ra, int32_t n_i)
{
    ugo_net* net = new ugo_net();
    net->n_ra = n_ra;
    net->n_i = n_i;
    net->num_steps = (int)(TRIAL_DURATION / TIMESTEP);
    net->ginh_res = 0.0;
    net->seed = 0;
    net->net_id = 0;
    std::memset(&net->syn, 0, sizeof(net->syn));
    std::memset(&net->mat, 0, sizeof(net->mat));
    std::memset(&net->noise, 0, sizeof(net->noise));
    std::memset(&net->conn, 0, sizeof(net->conn));
    net->ra.resize(n_ra);
    net->in.resize(n_i);
    for (auto& s : net->ra) ra_set_to_rest(s);
    net->ra2i.assign(n_ra, Conn());
    net->i2ra.assign(n_i, Conn());
    size_t nn = (size_t)n_ra * n_ra;
    net->W.assign(nn, 0.0); net->D.assign(nn, 0.0); net->L.assign(nn, 0.0);
    net->active.assign(nn, 0); net->super.assign(nn, 0);
    net->active_list.assign(n_ra, std::vector<int>());
    net->super_list.assign(n_ra, std::vector<int>());
    net->remodeled.assign(n_ra, 0); net->mature.assign(n_ra, 0); net->trials_after_replacement.assign(n_ra, 0);
    net->rest_potential.assign(n_ra, -80.0); net->gca.assign(n_ra, 55.0);
    net->maturation_scale.assign(n_ra, MATURATION_SCALE_SPONTANEOUS);
    net->firing_rate_long.assign(n_ra, 0.0);
    net->spread.assign(n_ra, 0.0);
    net->ra_xyz.assign((size_t)3 * n_ra, 0.0);
    net->i_xyz.assign((size_t)3 * n_i, 0.0);
    net->mean_injection_time = 0.0;
    net->log_deliveries = false;
    return net;
}

void ugo_free(ugo_net* net)
{
    if (net->gate_worker.joinable()) ugo_trial_end(net);
    delete net;
}

void ugo_set_params(ugo_net* net, const ugo_synaptic_params* syn, const ugo_maturation_params* mat,
                    const ugo_noise_params* noise, const ugo_connection_params* conn)
{
    net->syn = *syn;
    net->mat = *mat;
    net->noise = *noise;
    net->conn = *conn;
    net->hist.assign(net->n_ra, std::vector<int>(std::max(mat->RATE_WINDOW_LONG, ROBUSTNESS_WINDOW), 0));
}

void ugo_set_seed(ugo_net* net, uint64_t seed, uint32_t net_id) { net->seed = seed; net->net_id = net_id; }
void ugo_set_num_steps(ugo_net* net, int32_t num_steps) { net->num_steps = num_steps; }

void ugo_set_ra2i(ugo_net* net, const int32_t* off, const int32_t* tgt, const double* w, const double* d, const double* len)
{
    set_csr(net->ra2i, net->n_ra, off, tgt, w, d, len);
}

void ugo_set_i2ra(ugo_net* net, const int32_t* off, const int32_t* tgt, const double* w, const double* d, const double* len)
{
    set_csr(net->i2ra, net->n_i, off, tgt, w, d, len);
}

void ugo_set_rara(ugo_net* net, const double* w, const double* d, const double* len)
{
    size_t nn = (size_t)net->n_ra * net->n_ra;
    net->W.assign(w, w + nn);
    net->D.assign(d, d + nn);
    if (len) net->L.assign(len, len + nn);
}

void ugo_set_synapse_lists(ugo_net* net, const int32_t* aoff, const int32_t* atgt, const int32_t* soff, const int32_t* stgt)
{
    const int N = net->n_ra;
    std::fill(net->active.begin(), net->active.end(), 0);
    std::fill(net->super.begin(), net->super.end(), 0);
    for (int i = 0; i < N; ++i) {
        net->active_list[i].assign(atgt + aoff[i], atgt + aoff[i + 1]);
        net->super_list[i].assign(stgt + soff[i], stgt + soff[i + 1]);
        for (int j : net->active_list[i]) net->active[(size_t)i * N + j] = 1;
        for (int j : net->super_list[i]) net->super[(size_t)i * N + j] = 1;
    }
}

void ugo_set_neuron_props(ugo_net* net, const double* rest, const double* gca, const int32_t* mature,
                          const double* scale, const int32_t* remodeled, const int32_t* tar)
{
    const int N = net->n_ra;
    net->rest_potential.assign(rest, rest + N);
    net->gca.assign(gca, gca + N);
    net->mature.assign(mature, mature + N);
    net->maturation_scale.assign(scale, scale + N);
    net->remodeled.assign(remodeled, remodeled + N);
    net->trials_after_replacement.assign(tar, tar + N);
}

void ugo_set_training(ugo_net* net, int32_t n_tr, const int32_t* ids, const double* spread)
{
    std::vector<std::pair<int, double>> tr;
    for (int k = 0; k < n_tr; ++k) tr.push_back(std::make_pair(ids[k], spread ? spread[k] : 0.0));
    net->training.clear();
    std::fill(net->spread.begin(), net->spread.end(), 0.0);
    for (auto& p : tr) {
        net->training.push_back(p.first);
        net->spread[p.first] = p.second;
    }
    std::sort(net->training.begin(), net->training.end());
}

void ugo_set_coordinates(ugo_net* net, const double* ra_xyz, const double* i_xyz)
{
    net->ra_xyz.assign(ra_xyz, ra_xyz + (size_t)3 * net->n_ra);
    net->i_xyz.assign(i_xyz, i_xyz + (size_t)3 * net->n_i);
}

void ugo_set_activity_history(ugo_net* net, const int32_t* hist)
{
    const int W = net->mat.RATE_WINDOW_LONG;
    for (int i = 0; i < net->n_ra; ++i) net->hist[i].assign(hist + (size_t)i * W, hist + (size_t)(i + 1) * W);
}

void ugo_set_inhibition_tracking(ugo_net* net, double resolution)
{
    net->ginh_res = resolution > 0 ? resolution : 0.0;
    net->ginh.clear();
}

int32_t ugo_get_inhibition(const ugo_net* net, double* out, int64_t capacity)
{
    if (net->ginh_res <= 0 || net->n_ra == 0) return 0;
    const int32_t points = (int32_t)(net->ginh.size() / (size_t)net->n_ra);
    if (out && capacity >= (int64_t)net->ginh.size()) std::memcpy(out, net->ginh.data(), net->ginh.size() * sizeof(double));
    return points;
}

void ugo_set_trace(ugo_net* net, int32_t nra, const int32_t* ra_ids, int32_t ni, const int32_t* i_ids)
{
    net->trace_ra.assign(ra_ids, ra_ids + nra);
    net->trace_i.assign(i_ids, i_ids + ni);
}

int64_t ugo_get_trace(const ugo_net* net, int32_t which, double* out, int64_t cap)
{
    const std::vector<double>& b = which == 0 ? net->trace_ra_buf : net->trace_i_buf;
    if (out) std::memcpy(out, b.data(), sizeof(double) * (size_t)std::min<int64_t>(cap, (int64_t)b.size()));
    return (int64_t)b.size();
}

void ugo_set_delivery_log(ugo_net* net, int32_t enabled) { net->log_deliveries = enabled != 0; }

int64_t ugo_get_delivery_log(const ugo_net* net, int32_t* out3, int64_t cap)
{
    int64_t n = (int64_t)net->delivery_log.size() / 3;
    if (out3) std::memcpy(out3, net->delivery_log.data(), sizeof(int32_t) * 3 * (size_t)std::min(n, cap));
    return n;
}

int32_t ugo_run_trial(ugo_net* net, int32_t kind, int32_t training, uint32_t trial_index)
{
    return run_trial(net, kind == 1, training != 0, trial_index);
}

int32_t ugo_trial_begin(ugo_net* net, int32_t kind, int32_t training, uint32_t trial_index)
{
    if (net->gate_worker.joinable()) return -2;
    {
        std::lock_guard<std::mutex> lk(net->gate_mu);
        net->gated = true;
        net->gate_until = 1;
        net->gate_at = 0;
        net->gate_done = false;
    }
    net->gate_worker = std::thread([=] {
        int rc = run_trial(net, kind == 1, training != 0, trial_index);
        std::lock_guard<std::mutex> lk(net->gate_mu);
        net->gate_rc = rc;
        net->gate_at = net->num_steps;
        net->gate_done = true;
        net->gate_cv.notify_all();
    });
    std::unique_lock<std::mutex> lk(net->gate_mu);
    net->gate_cv.wait(lk, [&] { return net->gate_at >= 1 || net->gate_done; });
    return 0;
}

int32_t ugo_trial_advance(ugo_net* net, int32_t n_steps)
{
    std::unique_lock<std::mutex> lk(net->gate_mu);
    if (!net->gated || net->gate_done) return 0;
    const int from = net->gate_at;
    net->gate_until = from + n_steps;
    net->gate_cv.notify_all();
    net->gate_cv.wait(lk, [&] { return net->gate_at >= net->gate_until || net->gate_done; });
    return (net->gate_done ? net->num_steps : net->gate_at) - from;
}

int32_t ugo_trial_end(ugo_net* net)
{
    {
        std::lock_guard<std::mutex> lk(net->gate_mu);
        net->gate_until = INT_MAX;
        net->gate_cv.notify_all();
    }
    if (net->gate_worker.joinable()) net->gate_worker.join();
    net->gated = false;
    return net->gate_rc;
}

int32_t ugo_after_growth_trial(ugo_net* net, uint32_t trial_index)
{
    for (int i = 0; i < net->n_ra; ++i) net->trials_after_replacement[i] += 1;
    std::vector<int> rep;
    check_neuron_activity(net, rep);
    update_maturation(net);
    net->replaced = rep;
    if (!rep.empty()) replace_neurons(net, rep, trial_index);
    /* setToRest_afterEpoch: the next trial restarts every neuron from rest
     * (run_trial does this when it initialises the trial's noise streams). */
    return (int32_t)rep.size();
}

void ugo_reset_after_test(ugo_net* net) { (void)net; }

int64_t ugo_get_spikes(const ugo_net* net, int32_t which, int32_t* neuron, int32_t* step, int64_t cap)
{
    const std::vector<int>* n = which == 0 ? &net->spk_soma_n : which == 1 ? &net->spk_dend_n : &net->spk_i_n;
    const std::vector<int>* s = which == 0 ? &net->spk_soma_s : which == 1 ? &net->spk_dend_s : &net->spk_i_s;
    int64_t cnt = (int64_t)n->size();
    int64_t m = std::min(cnt, cap);
    if (neuron) std::memcpy(neuron, n->data(), sizeof(int32_t) * (size_t)m);
    if (step) std::memcpy(step, s->data(), sizeof(int32_t) * (size_t)m);
    return cnt;
}

double ugo_mean_injection_time(const ugo_net* net) { return net->mean_injection_time; }
double ugo_step_time(const ugo_net* net, int32_t step) { return net->T.empty() ? 0.0 : net->T[step]; }

void ugo_get_weights(const ugo_net* net, double* out) { std::memcpy(out, net->W.data(), sizeof(double) * net->W.size()); }
void ugo_get_delays(const ugo_net* net, double* out) { std::memcpy(out, net->D.data(), sizeof(double) * net->D.size()); }

int64_t ugo_get_list(const ugo_net* net, int32_t which, int32_t* off, int32_t* tgt)
{
    const std::vector<std::vector<int>>& L = which == 0 ? net->active_list : net->super_list;
    int64_t total = 0;
    for (int i = 0; i < net->n_ra; ++i) {
        if (off) off[i] = (int32_t)total;
        if (tgt) for (size_t k = 0; k < L[i].size(); ++k) tgt[total + (int64_t)k] = L[i][k];
        total += (int64_t)L[i].size();
    }
    if (off) off[net->n_ra] = (int32_t)total;
    return total;
}

void ugo_get_neuron_props(const ugo_net* net, double* rest, double* gca, int32_t* mature, double* scale,
                          int32_t* remodeled, int32_t* tar, double* frl)
{
    const int N = net->n_ra;
    for (int i = 0; i < N; ++i) {
        if (rest) rest[i] = net->rest_potential[i];
        if (gca) gca[i] = net->gca[i];
        if (mature) mature[i] = net->mature[i];
        if (scale) scale[i] = net->maturation_scale[i];
        if (remodeled) remodeled[i] = net->remodeled[i];
        if (tar) tar[i] = net->trials_after_replacement[i];
        if (frl) frl[i] = net->firing_rate_long[i];
    }
}

int64_t ugo_get_connections(const ugo_net* net, int32_t which, int32_t* off, int32_t* tgt, double* w, double* d)
{
    const std::vector<Conn>& C = which == 0 ? net->ra2i : net->i2ra;
    int64_t total = 0;
    for (size_t i = 0; i < C.size(); ++i) {
        if (off) off[i] = (int32_t)total;
        for (size_t k = 0; k < C[i].tgt.size(); ++k) {
            if (tgt) tgt[total + (int64_t)k] = C[i].tgt[k];
            if (w) w[total + (int64_t)k] = C[i].w[k];
            if (d) d[total + (int64_t)k] = C[i].d[k];
        }
        total += (int64_t)C[i].tgt.size();
    }
    if (off) off[C.size()] = (int32_t)total;
    return total;
}

void ugo_get_coordinates(const ugo_net* net, double* ra_xyz, double* i_xyz)
{
    if (ra_xyz) std::memcpy(ra_xyz, net->ra_xyz.data(), sizeof(double) * net->ra_xyz.size());
    if (i_xyz) std::memcpy(i_xyz, net->i_xyz.data(), sizeof(double) * net->i_xyz.size());
}

int64_t ugo_get_replaced(const ugo_net* net, int32_t* out, int64_t cap)
{
    int64_t n = (int64_t)net->replaced.size();
    if (out) for (int64_t k = 0; k < std::min(n, cap); ++k) out[k] = net->replaced[(size_t)k];
    return n;
}

void ugo_ra_single(int32_t n_steps, double Erest, double GCa, const ugo_noise_params* noise, uint64_t seed,
                   uint32_t trial, uint32_t neuron, const int32_t* kick_step, const double* kick_exc,
                   const double* kick_inh, int32_t n_kicks, double* trace_out, uint8_t* fired_out)
{
    RAState s;
    ra_set_to_rest(s);
    RAParams p;
    p.EL = Erest; p.GdCa = GCa;
    p.mu_s = noise->white_noise_mean_soma; p.sigma_s = noise->white_noise_std_soma;
    p.mu_d = noise->white_noise_mean_dend; p.sigma_d = noise->white_noise_std_dend;
    p.dt = TIMESTEP;
    ugo_stream st;
    ugo_stream_init(&st, seed, UGO_KIND_RA_WHITE, 0, neuron, trial);
    int kk = 0;
    for (int t = 0; t < n_steps; ++t) {
        while (kk < n_kicks && kick_step[kk] == t) {
            s.Gexc_d += kick_exc[kk];
            s.Ginh_d += kick_inh[kk];
            ++kk;
        }
        ra_step(s, p, st);
        double row[10] = { s.Vs, s.Vd, s.n, s.h, s.l, s.r, s.c, s.Ca, s.Gexc_d, s.Ginh_d };
        std::memcpy(trace_out + (size_t)t * 10, row, sizeof(row));
        fired_out[2 * t] = s.fired_soma ? 1 : 0;
        fired_out[2 * t + 1] = s.fired_dend ? 1 : 0;
    }
}

void ugo_i_single(int32_t n_steps, uint64_t seed, uint32_t trial, uint32_t neuron, const int32_t* kick_step,
                  const double* kick_exc, const double* kick_inh, int32_t n_kicks, double* trace_out, uint8_t* fired_out)
{
    IState s;
    ugo_stream st;
    ugo_stream_init(&st, seed, UGO_KIND_I_POISSON, 0, neuron, trial);
    i_set_to_rest(s, st, TIMESTEP);
    int kk = 0;
    for (int t = 0; t < n_steps; ++t) {
        while (kk < n_kicks && kick_step[kk] == t) {
            s.Gexc += kick_exc[kk];
            s.Ginh += kick_inh[kk];
            ++kk;
        }
        i_step(s, TIMESTEP, st);
        double row[7] = { s.V, s.n, s.m, s.h, s.w, s.Gexc, s.Ginh };
        std::memcpy(trace_out + (size_t)t * 7, row, sizeof(row));
        fired_out[t] = s.fired ? 1 : 0;
    }
}

void ugo_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { ugo_philox4x32_10(ctr, key, out); }

} // extern "C"
