// Single-precision HVC(RA) Debrabant step for two neurons per thread.
//
// Same equations as the reference's HH2_test (c++/src/HH2_test.cpp:613-754,
// RHS :866-890, gating c++/include/HH2_test.h:265-276), laid out for the
// Blackwell issue budget:
//  * every add/mul/fma works on the neuron pair with one f32x2 instruction;
//  * exponentials are MUFU ex2 with log2(e) folded into the affine argument;
//  * the seven reciprocals of a stage (mInf, nInf/tauN, lInf, hInf/tauH, rInf,
//    cInf and ca/(ca+6)) come from two MUFU rcp: 1/a = b/(ab) etc.
//  * (x - c) k products are single multiply-adds with the constants folded in.
// Per neuron and step: 32 ex2 + 8 rcp on the SFU.
#pragma once
#include "ug_neuron.cuh"

namespace ug {

__device__ __forceinline__ float mufu_ex2(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float mufu_rcp(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

typedef float2 f2;
__device__ __forceinline__ f2 S(float s) { return make_float2(s, s); }
__device__ __forceinline__ f2 operator+(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 operator-(f2 a, f2 b) { return __ffma2_rn(b, S(-1.0f), a); }
__device__ __forceinline__ f2 operator*(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ f2 ex2x2(f2 a) { return make_float2(mufu_ex2(a.x), mufu_ex2(a.y)); }
__device__ __forceinline__ f2 rcpx2(f2 a) { return make_float2(mufu_rcp(a.x), mufu_rcp(a.y)); }

struct RA2 { f2 Vs, Vd, n, h, l, r, c, Ca; };

// log2(e)-scaled affine arguments: exp(k (v + b)) = ex2(K v + K b), K = k log2 e
#define UG_L2E 1.4426950408889634
#define UG_EXA(k) ((float)((k) * UG_L2E))
#define UG_EXB(k, b) ((float)((k) * (b) * UG_L2E))

struct RAPair {
    f2 EL, GdCa;       // per-neuron parameters
    f2 mus, mud;       // 100000 mu / A
    f2 cs, cd;         // GsL EL + mus and GdL EL + mud: the constant parts of the leak terms
};

// The per-neuron constants of a pair.
__device__ __forceinline__ RAPair ra_pair(f2 EL, f2 GdCa, float mus, float mud)
{
    typedef RAConst K;
    RAPair P;
    P.EL = EL;
    P.GdCa = GdCa;
    P.mus = S(mus);
    P.mud = S(mud);
    P.cs = fma2(EL, S((float)K::GsL), S(mus));
    P.cd = fma2(EL, S((float)K::GdL), S(mud));
    return P;
}

__device__ __forceinline__ RA2 ra_rhs_x2(const RA2& y, f2 Ge, f2 Gi, const RAPair& P)
{
    typedef RAConst K;
    const f2 vs = y.Vs, vd = y.Vd;
    // gating exponentials (HH2_test.h:265-276)
    const f2 Em = ex2x2(fma2(vs, S(UG_EXA(-1.0 / 9.5)), S(UG_EXB(-1.0 / 9.5, 30.0))));
    const f2 En = ex2x2(fma2(vs, S(UG_EXA(-0.1)), S(UG_EXB(-0.1, 35.0))));
    const f2 Et = ex2x2(fma2(vs, S(UG_EXA(1.0 / 15.0)), S(UG_EXB(1.0 / 15.0, 27.0))));
    const f2 El = ex2x2(fma2(vs, S(UG_EXA(-0.2)), S(UG_EXB(-0.2, 40.0))));
    const f2 Eh = ex2x2(fma2(vs, S(UG_EXA(1.0 / 7.0)), S(UG_EXB(1.0 / 7.0, 45.0))));
    const f2 Eth = ex2x2(fma2(vs, S(UG_EXA(1.0 / 6.0)), S(UG_EXB(1.0 / 6.0, 40.5))));
    const f2 Er = ex2x2(fma2(vd, S(UG_EXA(-0.1)), S(UG_EXB(-0.1, 5.0))));
    const f2 Ec = ex2x2(fma2(vd, S(UG_EXA(-1.0 / 7.0)), S(UG_EXB(-1.0 / 7.0, -10.0))));
    // denominators
    const f2 Dm = Em + S(1.0f);
    const f2 an = En + S(1.0f), bn = Et + S(1.0f);
    const f2 Dn = an * fma2(bn, S(0.1f), S(0.5f));            // (1+En)(0.1(1+Et) + 0.5)
    const f2 Dl = El + S(1.0f);
    const f2 ah = Eh + S(1.0f), bh = Eth + S(1.0f);
    const f2 Dh = ah * fma2(bh, S(0.1f), S(0.75f));
    const f2 Dr = Er + S(1.0f);
    const f2 Dc = Ec + S(1.0f);
    const f2 Dca = y.Ca + S(6.0f);
    // group A: 1/Dm, 1/Dn, 1/Dl from one reciprocal
    const f2 pmn = Dm * Dn;
    const f2 rA = rcpx2(pmn * Dl);
    const f2 iDl = pmn * rA;
    const f2 rmn = Dl * rA;
    const f2 iDm = Dn * rmn, iDn = Dm * rmn;
    // group B: 1/Dh, 1/Dr, 1/Dc, 1/Dca from one reciprocal
    const f2 phr = Dh * Dr, pcc = Dc * Dca;
    const f2 rB = rcpx2(phr * pcc);
    const f2 rhr = pcc * rB, rcc = phr * rB;
    const f2 iDh = Dr * rhr, iDr = Dh * rhr, iDc = Dca * rcc, iDca = Dc * rcc;

    RA2 k;
    const f2 m = iDm;
    const f2 m3 = m * m * m;
    const f2 n2 = y.n * y.n;
    const f2 n4 = n2 * n2;
    // kVs = GsL (EL - vs) + GsNa m^3 h (EsNa - vs) + (GsK n^4 + GsKLT l)(EsK - vs) + mus
    //       + (vd - vs) 100000 / (Rc As); every (x - c) k is one multiply-add
    f2 t = fma2(vs, S(-(float)K::GsL), P.cs);
    t = fma2(m3 * y.h, fma2(vs, S(-(float)K::GsNa), S((float)(K::GsNa * K::EsNa))), t);
    t = fma2(fma2(n4, S((float)K::GsK), y.l * S((float)K::GsKLT)), S((float)K::EsK) - vs, t);
    k.Vs = fma2(vd - vs, S((float)(100000.0 / (K::Rc * K::As))), t);
    // kVd = GdL (EL - vd) + GdCa r^2 (EdCa - vd) - GdCaK (vd - EdK) c ca / (ca + 6)
    //       - Ge vd + Gi (Egaba - vd) + mud + (vs - vd) 100000 / (Rc Ad)
    const f2 gr2 = P.GdCa * y.r * y.r;
    const f2 eca = S((float)K::EdCa) - vd;
    f2 u = fma2(vd, S(-(float)K::GdL), P.cd);
    u = fma2(gr2, eca, u);
    u = fma2((vd - S((float)K::EdK)) * y.c, y.Ca * iDca * S(-(float)K::GdCaK), u);
    u = fma2(Ge + Gi, S(0.0f) - vd, fma2(Gi, S((float)K::Egaba), u));
    k.Vd = fma2(vs - vd, S((float)(100000.0 / (K::Rc * K::Ad))), u);
    // kn = (nInf - n)/tauN = (1 - n an) bn / Dn ; kh likewise
    k.n = fma2(y.n * S(-1.0f), an, S(1.0f)) * bn * iDn;
    k.h = fma2(y.h * S(-1.0f), ah, S(1.0f)) * bh * iDh;
    k.l = (iDl - y.l) * S(0.1f);
    k.r = iDr - y.r;
    k.c = (iDc - y.c) * S(1.0f / 15.0f);
    k.Ca = fma2(gr2, eca * S(0.1f), y.Ca * S(-0.02f));
    return k;
}

#define UG_RA2_FOR(M) M(Vs) M(Vd) M(n) M(h) M(l) M(r) M(c) M(Ca)

// One Debrabant step of two neurons; J* are the point-distribution values.
__device__ __forceinline__ void ra_debrabant_x2(RA2& s, f2& Ge, f2& Gi, const RAPair& P, const RAStep<float>& p,
                                                f2 J1s, f2 J2s, f2 J1d, f2 J2d)
{
    typedef RAConst K;
    const f2 dt = S(p.dt);
    const f2 ns = S(p.sq * p.sig_s * (float)(1.0 / (K::As * K::cm)));
    const f2 nd = S(p.sq * p.sig_d * (float)(1.0 / (K::Ad * K::cm)));
    const f2 Ge1 = Ge * S(p.e1), Gi1 = Gi * S(p.e1), Ge2 = Ge * S(p.e2), Gi2 = Gi * S(p.e2);

    // the noise amplitudes times the step's point values, once per step
    const f2 a1s = ns * J1s, a2s = ns * J2s, a1d = nd * J1d, a2d = nd * J2d;
    RA2 y = s;
    y.Vs = fma2(a1s, S(-0.01844540496323970f), fma2(a2s, S(-0.1866426386543421f), s.Vs));
    y.Vd = fma2(a1d, S(-0.01844540496323970f), fma2(a2d, S(-0.1866426386543421f), s.Vd));
    const RA2 a1 = ra_rhs_x2(y, Ge, Gi, P);

    RA2 h4, up;   // running sums of stage 4's increment and of the update
#define M(f) h4.f = a1.f * S(-0.4526683126055039f); up.f = a1.f * S(1.0f / 6.0f); y.f = fma2(dt, a1.f, s.f);
    UG_RA2_FOR(M)
#undef M
    y.Vs = fma2(a1s, S(0.8017012756521233f), fma2(a2s, S(-0.8575745885712401f), y.Vs));
    y.Vd = fma2(a1d, S(0.8017012756521233f), fma2(a2d, S(-0.8575745885712401f), y.Vd));
    const RA2 a2 = ra_rhs_x2(y, Ge1, Gi1, P);

    const f2 d8 = S(p.dt * 0.125f);
#define M(f) h4.f = fma2(a2.f, S(-0.4842227708685013f), h4.f); up.f = fma2(a2.f, S(-0.005430430675258792f), up.f); \
             y.f = fma2(d8, fma2(a1.f, S(3.0f), a2.f), s.f);
    UG_RA2_FOR(M)
#undef M
    y.Vs = fma2(a1s, S(0.5092227024816198f), fma2(a2s, S(-0.4723392695015512f), y.Vs));
    y.Vd = fma2(a1d, S(0.5092227024816198f), fma2(a2d, S(-0.4723392695015512f), y.Vd));
    const RA2 a3 = ra_rhs_x2(y, Ge2, Gi2, P);

#define M(f) h4.f = fma2(a3.f, S(1.9368910834740051f), h4.f); up.f = fma2(a3.f, S(2.0f / 3.0f), up.f); \
             y.f = fma2(dt, h4.f, s.f);
    UG_RA2_FOR(M)
#undef M
    y.Vs = fma2(a1s, S(0.9758794209767762f), fma2(a2s, S(0.3060354860326548f), y.Vs));
    y.Vd = fma2(a1d, S(0.9758794209767762f), fma2(a2d, S(0.3060354860326548f), y.Vd));
    const RA2 a4 = ra_rhs_x2(y, Ge1, Gi1, P);

#define M(f) s.f = fma2(dt, fma2(a4.f, S(0.1720970973419255f), up.f), s.f);
    UG_RA2_FOR(M)
#undef M
    s.Vs = fma2(a1s, S(100000.0f), s.Vs);
    s.Vd = fma2(a1d, S(100000.0f), s.Vd);
    Ge = Ge1;
    Gi = Gi1;
}

__device__ __forceinline__ Philox4 philox_wide(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0,
                                               uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return Philox4{c0, c1, c2, c3};
}

// The noise value of a word: the 30-point distribution index is (u * 30) >> 32, and
// index >= k exactly when u >= ceil(k 2^32 / 30), so unsigned comparisons against those
// bounds pick the value without a multiply.
__device__ __forceinline__ float ra_point_f(uint32_t u)
{
    return u < 143165577u ? 2.4494897f : u < 286331154u ? -2.4494897f : u < 1574821342u ? 1.0f
                                                                   : u < 2863311531u ? -1.0f : 0.0f;
}

// Philox4x32-10 with the key schedule precomputed (RAStep::ks): the round keys come from
// the kernel's parameters, so no instruction updates them.
__device__ __forceinline__ Philox4 philox_sched(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                                const uint32_t* ks)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ ks[2 * r];
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ ks[2 * r + 1];
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
    }
    return Philox4{c0, c1, c2, c3};}

}  // namespace ug
