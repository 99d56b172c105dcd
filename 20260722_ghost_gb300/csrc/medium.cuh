// medium.cuh -- complex wave numbers k = k_r + j k_i (k_i <= 0: a lossy
// medium, the causal branch of bor_solver.py:161-172) for the FP64 fills of a
// penetrable body's interior.  Plain C++ as well, so the host can replay these
// expressions against the oracle.
//
//   e^{-j k R} = e^{k_i R} (cos k_r R - j sin k_r R)
//   g(R) = e^{-j k R} / R,   p(R) = (1 + j k R) e^{-j k R} / R^3
//   1 / k^2 = conj(k)^2 / |k|^4
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define GB_HD_CK __host__ __device__ __forceinline__
#else
#define GB_HD_CK inline
#endif

namespace gb {

// e^{-j k R} / R times amp; out = (re, im)
GB_HD_CK void ck_green(double R, double kr, double ki, double amp, double *out)
{
    const double a = amp * exp(ki * R) / R;
    const double ph = kr * R;
    out[0] = a * cos(ph);
    out[1] = -a * sin(ph);
}

// (1 + j k R) e^{-j k R} / R^3 times amp: (1 - k_i R + j k_r R) e^{k_i R} (cos - j sin) / R^3
GB_HD_CK void ck_bracket(double R, double kr, double ki, double amp, double *out)
{
    const double a = amp * exp(ki * R) / (R * R * R);
    const double ph = kr * R, c = cos(ph), s = sin(ph);
    const double u = 1.0 - ki * R, v = kr * R;
    out[0] = a * (u * c + v * s);
    out[1] = a * (v * c - u * s);
}

// 1 / k^2
GB_HD_CK void ck_inv_k2(double kr, double ki, double *out)
{
    const double n2 = kr * kr + ki * ki;
    const double n4 = n2 * n2;
    out[0] = (kr * kr - ki * ki) / n4;
    out[1] = -2.0 * kr * ki / n4;
}

}  // namespace gb
