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
// error reporting helpers (host)
// ----------------------------------------------------------------------------
void set_last_error(const char *msg);
int check_launch(const char *where);

}  // namespace gb
