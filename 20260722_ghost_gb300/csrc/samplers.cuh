// samplers.cuh -- azimuth samplers of the modal kernels (sm_103a).
//
//   GreenSampler    g(R) = e^{-j k R} / R                 (EFIE; 1/(4 pi) in the tables)
//   BracketSampler  p(R) = (1 + j k R) e^{-j k R} / R^3   (MFIE brackets; idem)
//
// with R^2 = d^2 + a^2 s2, s2 = sin^2(xi/2), d^2 = (rho - rho')^2 + (z - z')^2
// and a^2 = 4 rho rho' (the C sampler's kernels, bor_stream_kernel.c:26-48 and
// 65-106).  The FP32 variants carry R^2, R and k R as double-float so that the
// phase is exact to ~1e-7 rad before an accurate sincosf.
#pragma once
#include "common.cuh"
#include "medium.cuh"

namespace gb {
namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;
// 2 pi = A + B + C; A (8 bits) and B (12 bits) are short enough that q*A and
// q*B are exact in FP32 for every reduction count q < 2^11 (k R < 12800).
constexpr float kTwoPiA = 6.28125f;
constexpr float kTwoPiB = 4059.0f / 2097152.0f;
constexpr float kTwoPiC = (float)(kTwoPi - 6.28125 - 4059.0 / 2097152.0);
constexpr float kInvTwoPi = (float)(1.0 / kTwoPi);

// d^2, a^2 and k split into (hi, lo) FP32 words
struct DfPair {
    float d2h, d2l, a2h, a2l, kh, kl;
    __device__ void init(double d2, double a2, double k) {
        d2h = (float)d2; d2l = (float)(d2 - (double)d2h);
        a2h = (float)a2; a2l = (float)(a2 - (double)a2h);
        kh = (float)k;   kl = (float)(k - (double)kh);
    }
};

// R = r + rl, k R = kr (+ small), and sin / cos of k R for one s2 = (hi, lo)
struct DfPhase {
    float r, rl, kr, sn, cs;
};

__device__ __forceinline__ DfPhase df_phase(const DfPair &P, float2 s2)
{
    DfPhase o;
    // R^2 = d^2 + a^2 s2 in double-float
    const float p = P.a2h * s2.x;
    const float pe = fmaf(P.a2h, s2.x, -p);
    const float t = P.d2h + p;
    const float bb = t - P.d2h;
    const float te = (P.d2h - (t - bb)) + (p - bb);
    const float lo = te + pe + fmaf(P.a2h, s2.y, P.a2l * s2.x) + P.d2l;
    const float R2 = t + lo;
    const float R2l = lo - (R2 - t);
    // R = r + rl from one rsqrt and one Newton-style correction
    const float rs = rsqrtf(R2);
    o.r = R2 * rs;
    const float e = fmaf(-o.r, o.r, R2) + R2l;
    o.rl = 0.5f * e * rs;
    // phase k R in double-float (ph + phl), reduced mod 2 pi: ph - q A is
    // exact, the subtraction of q B is made exact with a two-sum, and the
    // remaining small terms form a first-order correction dt.
    const float ph = P.kh * o.r;
    const float phe = fmaf(P.kh, o.r, -ph);
    const float phl = phe + fmaf(P.kh, o.rl, P.kl * o.r);
    const float q = rintf(ph * kInvTwoPi);
    const float t1 = fmaf(-q, kTwoPiA, ph);
    const float qb = -q * kTwoPiB;
    const float t2 = t1 + qb;
    const float tb = t2 - t1;
    const float t2e = (t1 - (t2 - tb)) + (qb - tb);
    const float dt = fmaf(-q, kTwoPiC, phl) + t2e;
    float sn, cs;
    sincosf(t2, &sn, &cs);
    o.sn = fmaf(dt, cs, sn);            // sin(t2 + dt)
    o.cs = fmaf(-dt, sn, cs);           // cos(t2 + dt)
    o.kr = ph + phl;
    return o;
}

template <class R> struct GreenSampler;

template <> struct GreenSampler<double> {
    using S2 = double;          // sin^2 table entry type
    double d2, a2, k;
    __device__ void init(double d2_, double a2_, double k_) { d2 = d2_; a2 = a2_; k = k_; }
    static __device__ __forceinline__ double load_s2(const double *t, int j) { return t[j]; }
    __device__ __forceinline__ double2 operator()(double s2) const {
        double R = sqrt(fma(a2, s2, d2));
        R = fmax(R, 1e-30);
        double sn, cs;
        sincos(k * R, &sn, &cs);
        const double amp = 1.0 / R;                  // 1/(4 pi) is folded into the tables
        return make_double2(amp * cs, -amp * sn);
    }
};

template <> struct GreenSampler<float> {
    using S2 = float2;          // (hi, lo) split of sin^2
    DfPair P;
    __device__ void init(double d2, double a2, double k) { P.init(d2, a2, k); }
    static __device__ __forceinline__ float2 load_s2(const double *t, int j) {
        const double v = t[j];
        const float hi = (float)v;
        return make_float2(hi, (float)(v - (double)hi));
    }
    __device__ __forceinline__ float2 operator()(float2 s2) const {
        const DfPhase ph = df_phase(P, s2);
        // 1/R = 1/(r + rl) from an IEEE reciprocal and a first-order correction
        const float ir = __frcp_rn(ph.r);
        const float amp = ir * fmaf(-ph.rl, ir, 1.0f);  // 1/(4 pi) is folded into the tables
        return make_float2(amp * ph.cs, -amp * ph.sn);
    }
};

// FP64 samplers with a complex wave number k_r + j k_i (lossy media)
struct GreenSamplerC {
    using S2 = double;
    double d2, a2, kr, ki;
    __device__ void init(double d2_, double a2_, double kr_, double ki_) { d2 = d2_; a2 = a2_; kr = kr_; ki = ki_; }
    static __device__ __forceinline__ double load_s2(const double *t, int j) { return t[j]; }
    __device__ __forceinline__ double2 operator()(double s2) const {
        const double R = fmax(sqrt(fma(a2, s2, d2)), 1e-30);
        double o[2];
        ck_green(R, kr, ki, 1.0, o);                 // 1/(4 pi) is folded into the tables
        return make_double2(o[0], o[1]);
    }
};

struct BracketSamplerC {
    using S2 = double;
    double d2, a2, kr, ki;
    __device__ void init(double d2_, double a2_, double kr_, double ki_) { d2 = d2_; a2 = a2_; kr = kr_; ki = ki_; }
    static __device__ __forceinline__ double load_s2(const double *t, int j) { return t[j]; }
    __device__ __forceinline__ double2 operator()(double s2) const {
        const double R = fmax(sqrt(fma(a2, s2, d2)), 1e-30);
        double o[2];
        ck_bracket(R, kr, ki, 1.0, o);
        return make_double2(o[0], o[1]);
    }
};

template <class R> struct BracketSampler;

template <> struct BracketSampler<double> {
    using S2 = double;
    double d2, a2, k;
    __device__ void init(double d2_, double a2_, double k_) { d2 = d2_; a2 = a2_; k = k_; }
    static __device__ __forceinline__ double load_s2(const double *t, int j) { return t[j]; }
    __device__ __forceinline__ double2 operator()(double s2) const {
        double R = sqrt(fma(a2, s2, d2));
        R = fmax(R, 1e-30);
        double sn, cs;
        const double kr = k * R;
        sincos(kr, &sn, &cs);
        const double ir = 1.0 / R;
        const double ir3 = ir * ir * ir;
        // (cos - j sin)(1 + j k R)
        return make_double2(fma(kr, sn, cs) * ir3, fma(kr, cs, -sn) * ir3);
    }
};

template <> struct BracketSampler<float> {
    using S2 = float2;
    DfPair P;
    __device__ void init(double d2, double a2, double k) { P.init(d2, a2, k); }
    static __device__ __forceinline__ float2 load_s2(const double *t, int j) {
        return GreenSampler<float>::load_s2(t, j);
    }
    __device__ __forceinline__ float2 operator()(float2 s2) const {
        const DfPhase ph = df_phase(P, s2);
        const float ir = __frcp_rn(ph.r);
        const float irc = ir * fmaf(-ph.rl, ir, 1.0f);
        const float ir3 = irc * irc * irc;
        return make_float2(fmaf(ph.kr, ph.sn, ph.cs) * ir3, fmaf(ph.kr, ph.cs, -ph.sn) * ir3);
    }
};

}  // namespace
}  // namespace gb
