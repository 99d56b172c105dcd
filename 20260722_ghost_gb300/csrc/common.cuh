// common.cuh -- shared device helpers for the GB300 BoR-MoM kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#include "../../include/ghost_bor.h"

#ifndef GB_PI
#define GB_PI 3.14159265358979323846
#endif

namespace gb {

// ----------------------------------------------------------------------------
// complex scalar types: interleaved (re, im) in float2 / double2
// ----------------------------------------------------------------------------
template <class R> struct cplx;
template <> struct cplx<float> { using T = float2; };
template <> struct cplx<double> { using T = double2; };
template <class R> using C = typename cplx<R>::T;

template <class R> __host__ __device__ __forceinline__ C<R> mk(R x, R y) { C<R> c; c.x = x; c.y = y; return c; }
template <class V> __host__ __device__ __forceinline__ V cadd(V a, V b) { a.x += b.x; a.y += b.y; return a; }
template <class V> __host__ __device__ __forceinline__ V csub(V a, V b) { a.x -= b.x; a.y -= b.y; return a; }
template <class V> __host__ __device__ __forceinline__ V cmul(V a, V b) {
    V c; c.x = a.x * b.x - a.y * b.y; c.y = a.x * b.y + a.y * b.x; return c;
}
template <class V, class S> __host__ __device__ __forceinline__ V cscale(V a, S s) { a.x *= s; a.y *= s; return a; }
// a + b*c (complex fused)
template <class V> __host__ __device__ __forceinline__ V cfma(V b, V c, V a) {
    a.x = fma(b.x, c.x, a.x); a.x = fma(-b.y, c.y, a.x);
    a.y = fma(b.x, c.y, a.y); a.y = fma(b.y, c.x, a.y);
    return a;
}
__device__ __forceinline__ float2 cfma(float2 b, float2 c, float2 a) {
    a.x = fmaf(b.x, c.x, a.x); a.x = fmaf(-b.y, c.y, a.x);
    a.y = fmaf(b.x, c.y, a.y); a.y = fmaf(b.y, c.x, a.y);
    return a;
}
// a - b*c
template <class V> __host__ __device__ __forceinline__ V cfms(V b, V c, V a) {
    b.x = -b.x; b.y = -b.y; return cfma(b, c, a);
}
template <class V> __host__ __device__ __forceinline__ auto cabs1(V a) -> decltype(a.x) {
    return fabs(a.x) + fabs(a.y);
}

// atomic accumulation of a complex value into global memory
__device__ __forceinline__ void catomic_add(float2 *p, float2 v) {
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
    atomicAdd(p, v);
#else
    atomicAdd(&p->x, v.x); atomicAdd(&p->y, v.y);
#endif
}
__device__ __forceinline__ void catomic_add(double2 *p, double2 v) {
    atomicAdd(&p->x, v.x); atomicAdd(&p->y, v.y);
}

// ----------------------------------------------------------------------------
// double-float arithmetic: a value is hi + lo with two FP32 words (~48 bits).
// Used where FP64-class accuracy is needed but FP64 throughput is not (the
// FP64 pipe of a GB300 runs at ~1/60 of the FP32 pipe).  Error-free
// transformations: TwoProd via fmaf, TwoSum (Knuth).
// ----------------------------------------------------------------------------
__device__ __forceinline__ float2 df_from(double x)
{
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}
__device__ __forceinline__ double df_to(float2 a) { return (double)a.x + (double)a.y; }

// s += a * b   (all double-float; s.y is left unnormalised, |s.y| << |s.x|)
__device__ __forceinline__ void df_mac(float2 &s, float2 a, float2 b)
{
    const float p = a.x * b.x;
    const float pe = fmaf(a.x, b.x, -p);
    const float t = s.x + p;
    const float bb = t - s.x;
    const float te = (s.x - (t - bb)) + (p - bb);
    s.y += te + pe + fmaf(a.x, b.y, a.y * b.x);
    s.x = t;
}

// a * b with a double-float and b double-float, renormalised result
__device__ __forceinline__ float2 df_mul(float2 a, float2 b)
{
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e += fmaf(a.x, b.y, a.y * b.x);
    const float h = p + e;
    return make_float2(h, e - (h - p));
}

// a + b, renormalised
__device__ __forceinline__ float2 df_add(float2 a, float2 b)
{
    const float s = a.x + b.x;
    const float bb = s - a.x;
    const float e = (a.x - (s - bb)) + (b.x - bb) + a.y + b.y;
    const float h = s + e;
    return make_float2(h, e - (h - s));
}

// ----------------------------------------------------------------------------
// packed FP32 pairs: the f32x2 instructions of sm_100+ do the same operation on
// both words of a 64-bit register pair, two lanes of work per instruction
// ----------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long p2_pk(float2 v)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(v.x), "f"(v.y));
    return r;
}
__device__ __forceinline__ float2 p2_up(unsigned long long r)
{
    float2 v;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(v.x), "=f"(v.y) : "l"(r));
    return v;
}
__device__ __forceinline__ float2 p2_fma(float2 a, float2 b, float2 c)
{
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(p2_pk(a)), "l"(p2_pk(b)), "l"(p2_pk(c)));
    return p2_up(d);
}
__device__ __forceinline__ float2 p2_add(float2 a, float2 b)
{
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(p2_pk(a)), "l"(p2_pk(b)));
    return p2_up(d);
}
__device__ __forceinline__ float2 p2_sub(float2 a, float2 b)
{
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(p2_pk(a)), "l"(p2_pk(b)));
    return p2_up(d);
}
__device__ __forceinline__ float2 p2_mul(float2 a, float2 b)
{
    unsigned long long d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(p2_pk(a)), "l"(p2_pk(b)));
    return p2_up(d);
}

__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, df_neg(b)); }
// complex double-float packed as (re.hi, re.lo, im.hi, im.lo)
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float4 f4(float2 re, float2 im) { return make_float4(re.x, re.y, im.x, im.y); }

// exact FP32 -> FP64 conversion by integer operations (ALU pipe): sign,
// rebiased exponent and the 23 fraction bits; zeros and subnormal inputs
// (below 1.2e-38) give 0
__device__ __forceinline__ double f2d_bits(float x)
{
    const unsigned u = __float_as_uint(x);
    const unsigned ex = (u >> 23) & 0xFFu;
    if (ex == 0u) return 0.0;
    const unsigned hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u & 0x7FFFFFu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}
// hi + lo of a double-float rounded to FP64: two integer conversions and one add
__device__ __forceinline__ double df_to_bits(float2 a) { return f2d_bits(a.x) + f2d_bits(a.y); }

// ----------------------------------------------------------------------------
// error reporting helpers (host)
// ----------------------------------------------------------------------------
void set_last_error(const char *msg);
int check_launch(const char *where);
// persistent grid size of the near-field kernels (CTAs) on the current device
int near_grid();

}  // namespace gb
