// brackets.cuh -- per point-pair coefficients of the bracket fills (MFIE
// n x grad G' and the IBC rotated principal-value term), shared by the far and
// near kernels of mfie_fill.cu.  Plain C++ as well, so the host can replay
// exactly these expressions against the oracle.
//
// With the test point at phi = 0, the source at phi' = -xi, d = (dr, dz) =
// test - source, s2 = sin^2(xi/2), t = (t_rho, t_z) the test tangent and t'
// the source tangent, every bracket is p(R) times {1, s2, sin(xi)} with
// per-pair coefficients, so three azimuth transforms of p -- C[p], C[p s2]
// (cosine) and S[p sin xi] (sine) -- give all four:
//   K_tt = c0 C[p] + c1 C[p s2],   K_ff = c2 C[p] + c3 C[p s2],
//   K_tf = -j c4 S,                K_ft = -j c5 S.
#pragma once

#if defined(__CUDACC__)
#define GB_HD __host__ __device__ __forceinline__
#else
#define GB_HD inline
#endif

namespace gb {

// MFIE brackets of the reference (bor_stream_kernel.c:65-106, bor_kernels.py:
// 273-306): F_tt = -p (c0' + c1' s2), F_ff = p (N0 - 2 s2 (N0 - rho' t_z)),
// F_tf = p sin(xi) dz, F_ft = -p sin(xi) e0 with N0 = t x d, X0 = t x t',
// A0 = t . d, D0 = t . t', c0' = d x t',
// c1' = 2 (A0 t_z t'_rho + t_rho rho' X0 + D0 t_z rho' + t_rho t'_rho N0),
// e0 = rho' X0 + t'_rho N0 (the s2^2 terms and, in F_ft, the s2 terms cancel).
GB_HD void mfie_bracket_coefs(double rp, double zp, double trp, double tzp,
                              double rq, double zq, double trq, double tzq, double *c)
{
    const double dr = rp - rq, dz = zp - zq;
    const double X0 = trp * tzq - tzp * trq;
    const double N0 = trp * dz - tzp * dr;
    const double A0 = trp * dr + tzp * dz;
    const double D0 = trp * trq + tzp * tzq;
    const double c0 = dr * tzq - dz * trq;
    const double c1 = 2.0 * (A0 * tzp * trq + trp * rq * X0 + D0 * tzp * rq + trp * trq * N0);
    const double e0 = rq * X0 + trq * N0;
    c[0] = -c0;
    c[1] = -c1;
    c[2] = N0;
    c[3] = -2.0 * (N0 - rq * tzp);
    c[4] = dz;
    c[5] = -e0;
}

// IBC rotated principal-value brackets B_uv = p W_u . [R x (n' x f_v)] with the
// source normal n' (bor_kernels.py:449-484, bor_stream_kernel.c:108-150):
//   B_tt = p (-N0 - 2 s2 (t_z rho - t_rho dz)),
//   B_ff = p (c0' + 2 s2 (t'_z rho' + t'_rho dz)),
//   B_tf = p sin(xi) (t_z t'_rho rho - t_rho t'_z rho' - t_rho t'_rho dz),
//   B_ft = p sin(xi) dz.
GB_HD void ibc_bracket_coefs(double rp, double zp, double trp, double tzp,
                             double rq, double zq, double trq, double tzq, double *c)
{
    const double dr = rp - rq, dz = zp - zq;
    c[0] = -(trp * dz - tzp * dr);
    c[1] = -2.0 * (tzp * rp - trp * dz);
    c[2] = dr * tzq - dz * trq;
    c[3] = 2.0 * (tzq * rq + trq * dz);
    c[4] = tzp * trq * rp - trp * tzq * rq - trp * trq * dz;
    c[5] = dz;
}

// Geometric factors f_uv of the four IBC brackets at one azimuth sample for the
// device sampler (the reference's per-sample form, bor_stream_kernel.c:108-150):
// test point (rho, z) with tangent t at phi = 0, source (rho', z') with tangent
// t' and outward normal n' = (-t'_z, t'_rho) at phi' = -xi, cx = cos xi,
// sx = sin xi, dz = z - z', D = rho cos xi - rho':
//   f_uv = (W_u . n')(R . f'_v) - (W_u . f'_v)(R . n'),  uv = tt, tf, ft, ff;
// the bracket sample is p(R) f_uv.
GB_HD void ibc_sample_factors(double rp, double rq, double dz, double trp, double tzp,
                              double trq, double tzq, double cx, double sx, double *f)
{
    const double wt_n = -trp * tzq * cx + tzp * trq;
    const double wf_n = tzq * sx;
    const double D = rp * cx - rq;
    const double r_t = trq * D + tzq * dz;
    const double r_f = rp * sx;
    const double r_n = -tzq * D + trq * dz;
    const double wt_t = trp * trq * cx + tzp * tzq;
    const double wt_f = trp * sx;
    const double wf_t = -trq * sx;
    const double wf_f = cx;
    f[0] = wt_n * r_t - wt_t * r_n;
    f[1] = wt_n * r_f - wt_f * r_n;
    f[2] = wf_n * r_t - wf_t * r_n;
    f[3] = wf_n * r_f - wf_f * r_n;
}

template <bool IBC>
GB_HD void bracket_coefs(double rp, double zp, double trp, double tzp,
                         double rq, double zq, double trq, double tzq, double *c)
{
    if (IBC)
        ibc_bracket_coefs(rp, zp, trp, tzp, rq, zq, trq, tzq, c);
    else
        mfie_bracket_coefs(rp, zp, trp, tzp, rq, zq, trq, tzq, c);
}

// The value a bracket fill adds to one block entry, from the kernel's four
// bracket sums K (tt, tf, ft, ff after the -j of the sine terms): the MFIE
// operator Z_M = M/2 - K takes -K, the IBC addition Z_s (M/2 + B) takes +K;
// the mass term (self pairs, diagonal blocks) enters with +1/2 in both.  The
// result is scaled by s = scale (MFIE) or scale * Z_s(source element) (IBC).
template <bool IBC>
GB_HD void bracket_entry(double kx, double ky, double mass_half, double s_re, double s_im,
                         double *out)
{
    const double vx = (IBC ? kx : -kx) + mass_half;
    const double vy = IBC ? ky : -ky;
    out[0] = s_re * vx - s_im * vy;
    out[1] = s_re * vy + s_im * vx;
}

}  // namespace gb
