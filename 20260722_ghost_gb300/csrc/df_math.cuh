// df_math.cuh -- double-float (two FP32 words, ~48 bits) elementary functions
// for the near-field node evaluation, so that the transcendental work of each
// azimuth node runs on the FP32 pipe (the FP64 pipe of a GB300 is ~1/64 of it).
//
//   df_rsqrt     1/sqrt(x): rsqrtf seed and one Newton step in double-float
//   df_reduce    k R  ->  t in [-pi, pi]: Cody-Waite reduction by a 4-word 2 pi
//   df_sincos    sin and cos of |t| <= 1.01 pi: table-driven (Tang's method),
//                t = j pi/128 + r with |r| <= pi/256, the table holding
//                sin, cos of j pi/128 as double-float, and short Taylor series
//                of sin r and cos r whose tails are small enough for FP32
//
// Accuracy: ~1e-14 absolute for sin/cos of a double-float argument; the phase
// k R carries the double-float relative error of k and R (~4e-15 k R).
#pragma once
#include "common.cuh"

namespace gb {
namespace {

// 2 pi = A + B + C + D: A (8 significant bits) and B (12) make q A and q B
// exact for reduction counts q < 2^11; C and D are FP32 roundings of the rest.
constexpr float kDfTwoPiA = 6.28125f;
constexpr float kDfTwoPiB = 4059.0f / 2097152.0f;
constexpr float kDfTwoPiC = -1.7484555314695172e-07f;
constexpr float kDfTwoPiD = -6.8604980400235275e-15f;
constexpr float kDfInvTwoPi = 0.15915493667125702f;
// pi / 128 = P1 + P2 + P3, P1 with 15 significant bits (j P1 exact for |j| <= 256)
constexpr float kDfPiB128_1 = 0.02454376220703125f;
constexpr float kDfPiB128_2 = -6.960085841001273e-08f;
constexpr float kDfPiB128_3 = -2.5803118085395652e-15f;
constexpr float kDf128ByPi = 40.7436637878418f;
constexpr int kDfTabN = 257;           // j = -128 .. 128
// ln 2 / 32 = L1 + L2 + L3, L1 with 13 significant bits (k L1 exact for k < 2^11)
constexpr float kDfLn2By32_1 = 0.02165985107421875f;
constexpr float kDfLn2By32_2 = 9.983182280848268e-07f;
constexpr float kDfLn2By32_3 = 5.14560928046269e-14f;
constexpr float kDf32ByLn2 = 46.16624069213867f;
constexpr int kDfExpTabN = 32;         // 2^(j/32), j = 0..31

__device__ __forceinline__ float2 df_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return make_float2(s, (a - (s - bb)) + (b - bb));
}
__device__ __forceinline__ float2 df_fast(float hi, float lo)    // |hi| >= |lo|
{
    const float s = hi + lo;
    return make_float2(s, lo - (s - hi));
}
// double-float times FP32
__device__ __forceinline__ float2 df_mulf(float2 a, float b)
{
    const float p = a.x * b;
    const float e = fmaf(a.x, b, -p) + a.y * b;
    return df_fast(p, e);
}

// table of sin, cos (j pi / 128), j = -128..128, as (sin hi, sin lo, cos hi, cos lo);
// filled cooperatively by a CTA (FP64 sincos, once per CTA)
__device__ __forceinline__ void df_fill_sincos_table(float4 *tab)
{
    for (int i = threadIdx.x; i < kDfTabN; i += blockDim.x) {
        double s, c;
        sincospi((double)(i - 128) / 128.0, &s, &c);
        const float2 sf = df_from(s), cf = df_from(c);
        tab[i] = make_float4(sf.x, sf.y, cf.x, cf.y);
    }
}

// table of 2^(j/32), j = 0..31, as double-float; filled cooperatively by a CTA
__device__ __forceinline__ void df_fill_exp_table(float2 *tab)
{
    for (int i = threadIdx.x; i < kDfExpTabN; i += blockDim.x) tab[i] = df_from(exp2((double)i / 32.0));
}

// 1 / a, a double-float, from an IEEE reciprocal and one Newton step
__device__ __forceinline__ float2 df_rcp(float2 a)
{
    const float y = __frcp_rn(a.x);
    const float p = a.x * y;
    const float pe = fmaf(a.x, y, -p);
    const float e = ((1.0f - p) - pe) - a.y * y;
    return df_fast(y, y * e);
}

// e^v and e^v - 1 for 0 <= v < 88 (double-float), Tang's table-driven method:
// v = (32 n + j) ln2/32 + r, |r| <= ln2/64, e^v = 2^n 2^(j/32) e^r with
// e^r - 1 = r + r^2/2 + r^3 (1/6 + r/24 + r^2/120 + r^3/720); e^v - 1 comes
// straight from the series when n = j = 0 (no cancellation for small v)
__device__ __forceinline__ void df_exp(float2 v, const float2 *__restrict__ tab, float2 &E, float2 &Em1)
{
    const float kf = rintf(v.x * kDf32ByLn2);
    const int k = (int)kf;
    const float r1 = fmaf(-kf, kDfLn2By32_1, v.x);        // exact
    const float p2 = kf * kDfLn2By32_2;
    const float p2e = fmaf(kf, kDfLn2By32_2, -p2);
    const float2 rs = df_two_sum(r1, -p2);
    const float2 r = df_fast(rs.x, rs.y - p2e - kf * kDfLn2By32_3 + v.y);
    const float rr = r.x * r.x;
    const float rre = fmaf(r.x, r.x, -rr) + 2.0f * r.x * r.y;
    const float c = r.x * fmaf(r.x, fmaf(r.x, fmaf(r.x, 1.0f / 720.0f, 1.0f / 120.0f), 1.0f / 24.0f), 1.0f / 6.0f);
    const float2 h = df_two_sum(r.x, 0.5f * rr);
    const float2 em1r = df_fast(h.x, h.y + r.y + 0.5f * rre + rr * c);
    if (k == 0) {
        Em1 = em1r;
        const float2 o = df_two_sum(1.0f, em1r.x);
        E = df_fast(o.x, o.y + em1r.y);
        return;
    }
    const float2 o = df_two_sum(1.0f, em1r.x);
    const float2 er = df_fast(o.x, o.y + em1r.y);
    const float2 t = df_mul(tab[k & 31], er);
    const float sc = __int_as_float(((k >> 5) + 127) << 23);     // 2^n, exact
    E = make_float2(t.x * sc, t.y * sc);
    Em1 = df_add(E, make_float2(-1.0f, 0.0f));
}

// 1 / sqrt(x), x > 0 double-float
__device__ __forceinline__ float2 df_rsqrt(float2 x)
{
    const float y = rsqrtf(x.x);
    // e = 1 - x y^2 from an exact y^2 and fused products (|e| ~ 1e-7)
    const float y2 = y * y;
    const float y2e = fmaf(y, y, -y2);
    const float p = x.x * y2;
    const float pe = fmaf(x.x, y2, -p);
    const float e = ((1.0f - p) - pe) - (x.x * y2e + x.y * y2);
    return df_fast(y, 0.5f * y * e);
}

// t = ph - q 2 pi (double-float), q = round(ph / 2 pi); |ph| < 2^11 * 2 pi
__device__ __forceinline__ float2 df_reduce(float2 ph)
{
    const float q = rintf(ph.x * kDfInvTwoPi);
    const float t1 = fmaf(-q, kDfTwoPiA, ph.x);          // exact
    const float t2 = fmaf(-q, kDfTwoPiB, t1);            // exact
    const float pc = q * kDfTwoPiC;
    const float pce = fmaf(q, kDfTwoPiC, -pc);
    const float2 s = df_two_sum(t2, -pc);
    // ph.y is bounded by half an ulp of ph.x (up to ~2^-13 here), so it joins
    // the high word through a two-sum before the small terms are added
    const float2 h = df_two_sum(s.x, ph.y);
    return df_fast(h.x, h.y + (s.y - pce - q * kDfTwoPiD));
}

// sin and cos of a double-float |t| <= 1.01 pi
__device__ __forceinline__ void df_sincos(float2 t, const float4 *__restrict__ tab, float2 &sn, float2 &cs)
{
    const int j = max(-128, min(128, (int)rintf(t.x * kDf128ByPi)));
    const float jf = (float)j;
    // r = t - j pi/128: the first step is exact, the second a two-product
    const float r1 = fmaf(-jf, kDfPiB128_1, t.x);
    const float p2 = jf * kDfPiB128_2;
    const float p2e = fmaf(jf, kDfPiB128_2, -p2);
    const float2 rs = df_two_sum(r1, -p2);
    const float2 r = df_fast(rs.x, rs.y - p2e - jf * kDfPiB128_3 + t.y);
    // r^2 as double-float
    const float rr = r.x * r.x;
    const float rre = fmaf(r.x, r.x, -rr) + 2.0f * r.x * r.y;
    // sin r = r + r^3 (-1/6 + r^2/120 - r^4/5040): the tail is < 3.1e-7
    const float st = r.x * rr * fmaf(rr, fmaf(rr, -1.0f / 5040.0f, 1.0f / 120.0f), -1.0f / 6.0f);
    const float2 sr = df_fast(r.x, r.y + st);
    // cos r = 1 - r^2/2 + r^4 (1/24 - r^2/720): the last term is < 9.6e-10
    const float c4 = rr * rr * fmaf(rr, -1.0f / 720.0f, 1.0f / 24.0f);
    const float2 ch = df_two_sum(1.0f, -0.5f * rr);
    const float2 cr = df_fast(ch.x, ch.y - 0.5f * rre + c4);
    const float4 T = tab[j + 128];
    const float2 sT = make_float2(T.x, T.y), cT = make_float2(T.z, T.w);
    // sin(a + r) = sin a cos r + cos a sin r;  cos(a + r) = cos a cos r - sin a sin r
    sn = df_add(df_mul(sT, cr), df_mul(cT, sr));
    const float2 m2 = df_mul(sT, sr);
    cs = df_add(df_mul(cT, cr), make_float2(-m2.x, -m2.y));
}

}  // namespace
}  // namespace gb
