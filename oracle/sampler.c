/*
 * oracle/sampler.c -- TEST INFRASTRUCTURE ONLY (the CPU oracle's sampler).
 *
 * Plain-C restatement of the reference's azimuthal integrand sampler
 * (bor_stream_kernel.c:26-48 sample_g, :51-63 pR, :65-106 sample_mfie) so the
 * NumPy oracle (oracle/bor_oracle.py) can time the reference algorithm on the
 * host at native speed.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU legs load this file's build; the GPU product never does.
 *
 * Layout: out[i][j][l] interleaved complex double, i < nr test points,
 * j < np_ source points, l < nxi azimuth samples xi_l = -pi + 2 pi l / nxi.
 *
 *   g(xi)      = exp(-j k R) / (4 pi R),  R^2 = d^2 + 4 rho rho' sin^2(xi/2)
 *   p(R)       = (1 + j k R) exp(-j k R) / (4 pi R^3)
 *   MFIE uv    = -p(R) [ (W_u . R)(n . f_v) - (W_u . f_v)(n . R) ]
 *
 * Coincident points are clamped to R = 1e-30 (the caller zeroes every
 * same/adjacent-element pair after the transform, as the reference does).
 */
#include <math.h>
#include <stddef.h>

#define ORACLE_R_MIN 1e-30
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

void oracle_sample_g(int nr, int np_, int nxi,
                     const double *rho_p, const double *z_p,
                     const double *rho_q, const double *z_q,
                     double k, const double *sin2_tab, double *out)
{
    for (int i = 0; i < nr; ++i) {
        const double rp = rho_p[i], zp = z_p[i];
        for (int j = 0; j < np_; ++j) {
            const double drho = rp - rho_q[j];
            const double dz = zp - z_q[j];
            const double dist2 = drho * drho + dz * dz;
            const double four_rr = 4.0 * rp * rho_q[j];
            double *dst = out + 2 * (size_t)nxi * ((size_t)i * np_ + j);
            for (int l = 0; l < nxi; ++l) {
                double R = sqrt(dist2 + four_rr * sin2_tab[l]);
                if (R < ORACLE_R_MIN) R = ORACLE_R_MIN;
                const double amp = 1.0 / (4.0 * M_PI * R);
                const double phase = k * R;
                dst[2 * l] = amp * cos(phase);
                dst[2 * l + 1] = -amp * sin(phase);
            }
        }
    }
}

static void oracle_p_of_r(double Rx, double Ry, double Rz, double k,
                          double *p_re, double *p_im)
{
    double R = sqrt(Rx * Rx + Ry * Ry + Rz * Rz);
    if (R < ORACLE_R_MIN) R = ORACLE_R_MIN;
    const double amp = 1.0 / (4.0 * M_PI * R * R * R);
    const double kr = k * R;
    const double c = cos(kr), s = sin(kr);
    /* (1 + j kR)(cos kR - j sin kR) */
    *p_re = amp * (c + kr * s);
    *p_im = amp * (kr * c - s);
}

void oracle_sample_mfie(int nr, int np_, int nxi,
                        const double *rho_p, const double *z_p,
                        const double *tr_p, const double *tz_p,
                        const double *rho_q, const double *z_q,
                        const double *tr_q, const double *tz_q,
                        double k, const double *cos_tab, const double *sin_tab,
                        double *o_tt, double *o_tf, double *o_ft, double *o_ff)
{
    for (int i = 0; i < nr; ++i) {
        for (int j = 0; j < np_; ++j) {
            const double Rz = z_p[i] - z_q[j];
            const size_t base = 2 * (size_t)nxi * ((size_t)i * np_ + j);
            for (int l = 0; l < nxi; ++l) {
                const double cx = cos_tab[l], sx = sin_tab[l];
                const double Rx = rho_p[i] - rho_q[j] * cx;
                const double Ry = rho_q[j] * sx;
                double pr, pi;
                oracle_p_of_r(Rx, Ry, Rz, k, &pr, &pi);
                /* test tangents W_t = (tr_p, 0, tz_p), W_f = (0, 1, 0);
                 * test normal n = (-tz_p, 0, tr_p); source at phi' = -xi. */
                const double WtR = tr_p[i] * Rx + tz_p[i] * Rz;
                const double WfR = Ry;
                const double nR = -tz_p[i] * Rx + tr_p[i] * Rz;
                const double n_tq = -tz_p[i] * tr_q[j] * cx + tr_p[i] * tz_q[j];
                const double n_fq = -tz_p[i] * sx;
                const double Wt_tq = tr_p[i] * tr_q[j] * cx + tz_p[i] * tz_q[j];
                const double Wt_fq = tr_p[i] * sx;
                const double Wf_tq = -tr_q[j] * sx;
                const double Wf_fq = cx;
                double f;
                f = -(WtR * n_tq - Wt_tq * nR);
                o_tt[base + 2 * l] = f * pr; o_tt[base + 2 * l + 1] = f * pi;
                f = -(WtR * n_fq - Wt_fq * nR);
                o_tf[base + 2 * l] = f * pr; o_tf[base + 2 * l + 1] = f * pi;
                f = -(WfR * n_tq - Wf_tq * nR);
                o_ft[base + 2 * l] = f * pr; o_ft[base + 2 * l + 1] = f * pi;
                f = -(WfR * n_fq - Wf_fq * nR);
                o_ff[base + 2 * l] = f * pr; o_ff[base + 2 * l + 1] = f * pi;
            }
        }
    }
}
