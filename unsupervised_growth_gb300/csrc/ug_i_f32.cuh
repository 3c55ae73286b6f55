// Single-precision HVC(I) DP8 step and the interneuron noise pre-pass.
//
// Equations of HHI_buffer (c++/src/HHI_buffer.cpp:426-690, rates
// c++/include/HHI_buffer.h:173-180), arranged for the SFU and issue budget:
//  * the three rates with slope -1/10 in v share one exponential:
//      E1 = exp(-(v+15)/10), exp(-(v+22)/10) = E1 e^-0.7, exp(-(v+4)/10) = E1 e^1.1,
//      and exp(-v/5) = (E1 e^1.5)^2;
//  * the four reciprocals of a stage (an, am, bh, wInf) come from one MUFU rcp;
//  * (V, n) and (m, h) travel as f32x2 pairs through the tableau sums.
// Per neuron and stage: 4 ex2 + 1 rcp (60 SFU operations per step).
//
// The Poisson noise of an interneuron does not depend on its state
// (HHI_buffer::noise_check, HHI_buffer.cpp:278-294 only compares the neuron's
// clock with the next noise time), so the single build draws every noise event
// of the trial before integrating: k_noise_events stores (step, conductance
// kick) pairs per channel, consuming the neuron's stream in the reference's
// order (exc before inh within a step).  The integrator then applies kicks at
// their steps with no double-precision work in its loop.
#pragma once
#include "ug_ra_f32x2.cuh"

namespace ug {

struct IK2 { f2 Vn, mh; float w; };

// x / (1 - exp(-x/10)) with E = exp(-x/10); near x = 0 the series 10 + x/2 + x^2/120
__device__ __forceinline__ float i_vtrap_den(float x, float E) { return fabsf(x) < 1e-3f ? 1.0f : 1.0f - E; }
__device__ __forceinline__ float i_vtrap_fin(float x, float inv) { return fabsf(x) < 1e-3f ? 10.0f + x * (0.5f + x * (1.0f / 120.0f)) : x * inv; }

__device__ __forceinline__ IK2 i_rhs_x(float v, f2 Vn, f2 mh, float w, float Ge, float Gi)
{
    typedef IConst K;
    const float E1 = mufu_ex2(fmaf(v, UG_EXA(-0.1), UG_EXB(-0.1, 15.0)));   // exp(-(v+15)/10)
    const float E2 = E1 * 0.49658530379140947f;                                  // exp(-(v+22)/10)
    const float Eb = E1 * 3.0041660239464334f;                                   // exp(-(v+4)/10)
    const float Ew0 = E1 * 4.4816890703380645f;                                  // exp(-v/10)
    const float Ew = Ew0 * Ew0;                                                  // exp(-v/5)
    const float Ebn = mufu_ex2(fmaf(v, UG_EXA(-1.0 / 80.0), UG_EXB(-1.0 / 80.0, 25.0)));
    const float Ebm = mufu_ex2(fmaf(v, UG_EXA(-1.0 / 18.0), UG_EXB(-1.0 / 18.0, 47.0)));
    const float Eah = mufu_ex2(fmaf(v, UG_EXA(-0.05), UG_EXB(-0.05, 34.0)));
    const float x1 = v + 15.0f, x2 = v + 22.0f;
    const float D1 = i_vtrap_den(x1, E1), D2 = i_vtrap_den(x2, E2);
    const float D3 = 1.0f + Eb, D4 = 1.0f + Ew;
    // four reciprocals from one
    const float p12 = D1 * D2, p34 = D3 * D4;
    const float r = mufu_rcp(p12 * p34);
    const float r12 = p34 * r, r34 = p12 * r;
    const float an = 0.15f * i_vtrap_fin(x1, D2 * r12);
    const float am = i_vtrap_fin(x2, D1 * r12);
    const float bh = 10.0f * (D4 * r34);
    const float wInf = D3 * r34;
    const float bn = 0.2f * Ebn, bm = 40.0f * Ebm, ah = 0.7f * Eah;
    IK2 k;
    const float n = Vn.y, m = mh.x, h = mh.y;
    const float n2 = n * n;
    const float m3 = m * m * m;
    float kv = -(float)K::gL * (v - (float)K::El);
    kv = fmaf(-(float)K::gNa * h * m3, v - (float)K::Ena, kv);
    kv = fmaf(-((float)K::gKdr * n2 * n2 + (float)K::gKHT * w), v - (float)K::Ek, kv);
    kv = fmaf(-Ge, v, kv);
    kv = fmaf(-Gi, v - (float)K::Ei, kv);
    // (kn, km) = (an, am)(1 - (n, m)) - (bn, bm)(n, m)
    const f2 nm = make_float2(n, m);
    const f2 knm = fma2(make_float2(an, am), S(1.0f) - nm, make_float2(-bn, -bm) * nm);
    k.Vn = make_float2(kv, knm.x);
    k.mh = make_float2(knm.y, fmaf(ah, 1.0f - h, -bh * h));
    k.w = wInf - w;
    return k;
}

// Conductance decay factors of the 12 stages (float build: constants).
__device__ __forceinline__ void i_dp8_x(IStateR<float>& s, const IStep<float>& p)
{
    const DPT B7[] = {UG_DP_B7}, B8[] = {UG_DP_B8}, B9[] = {UG_DP_B9}, B10[] = {UG_DP_B10}, B11[] = {UG_DP_B11},
              B12[] = {UG_DP_B12}, BO[] = {UG_DP_OUT};
    const DPT* tb[6] = {B7, B8, B9, B10, B11, B12};
    const int cnt[6] = {4, 5, 6, 7, 8, 9};
    const int acount[5] = {1, 2, 2, 3, 3};
    const int astage[5][3] = {{0, 0, 0}, {0, 1, 0}, {0, 2, 0}, {0, 2, 3}, {0, 3, 4}};
    const double acoef[5][3] = {{1, 0, 0}, {1, 3, 0}, {1, 3, 0}, {20, -75, 75}, {3, 15, 12}};
    const double aden[5] = {18, 48, 32, 64, 80};
    const f2 dt2 = S(p.dt);
    const f2 Vn0 = make_float2(s.V, s.n), mh0 = make_float2(s.m, s.h);
    f2 kVn[12], kmh[12];
    float kw[12];
#pragma unroll
    for (int st = 0; st < 12; ++st) {
        f2 Vn = Vn0, mh = mh0;
        float w = s.w;
        if (st > 0) {
            f2 aVn = S(0.f), amh = S(0.f);
            float aw = 0.f;
            if (st <= 5) {
                const int a = st - 1;
#pragma unroll
                for (int j = 0; j < 3; ++j) {
                    if (j < acount[a]) {
                        const int q = astage[a][j];
                        const float c = (float)(acoef[a][j] / aden[a]);
                        aVn = fma2(kVn[q], S(c), aVn);
                        amh = fma2(kmh[q], S(c), amh);
                        aw = fmaf(kw[q], c, aw);
                    }
                }
            } else {
                const DPT* t = tb[st - 6];
#pragma unroll
                for (int j = 0; j < 9; ++j) {
                    if (j < cnt[st - 6]) {
                        const int q = t[j].s;
                        const float c = (float)(t[j].num / t[j].den);
                        aVn = fma2(kVn[q], S(c), aVn);
                        amh = fma2(kmh[q], S(c), amh);
                        aw = fmaf(kw[q], c, aw);
                    }
                }
            }
            Vn = fma2(dt2, aVn, Vn0);
            mh = fma2(dt2, amh, mh0);
            w = fmaf(p.dt, aw, s.w);
        }
        const IK2 k = i_rhs_x(Vn.x, Vn, mh, w, s.Ge * p.ge[st], s.Gi * p.gi[st]);
        kVn[st] = k.Vn;
        kmh[st] = k.mh;
        kw[st] = k.w;
    }
    f2 oVn = S(0.f), omh = S(0.f);
    float ow = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int q = BO[j].s;
        const float c = (float)(BO[j].num / BO[j].den);
        oVn = fma2(kVn[q], S(c), oVn);
        omh = fma2(kmh[q], S(c), omh);
        ow = fmaf(kw[q], c, ow);
    }
    const f2 Vn = fma2(dt2, oVn, Vn0), mh = fma2(dt2, omh, mh0);
    s.V = Vn.x;
    s.n = Vn.y;
    s.m = mh.x;
    s.h = mh.y;
    s.w = fmaf(p.dt, ow, s.w);
    s.Ge = s.Ge * p.ge[11];
    s.Gi = s.Gi * p.gi[11];
}

}  // namespace ug
