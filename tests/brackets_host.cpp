// Host build of the bracket-fill coefficient code (csrc/brackets.cuh) for the
// CPU tests: the same expressions the MFIE and IBC fill kernels compile.
#include <cmath>
#include <cstddef>

#include "brackets.cuh"

extern "C" {

// pairs [n][8] = (rho, z, t_rho, t_z) of the test point, then of the source
// point; out [n][6] = c0..c5
void host_bracket_coefs(int ibc, int n, const double *pairs, double *out)
{
    for (int i = 0; i < n; ++i) {
        const double *q = pairs + 8 * i;
        if (ibc)
            gb::bracket_coefs<true>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], out + 6 * i);
        else
            gb::bracket_coefs<false>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], out + 6 * i);
    }
}

// in [n][5] = (K re, K im, mass/2, scale re, scale im); out [n][2]
void host_bracket_entry(int ibc, int n, const double *in, double *out)
{
    for (int i = 0; i < n; ++i) {
        const double *v = in + 5 * i;
        if (ibc)
            gb::bracket_entry<true>(v[0], v[1], v[2], v[3], v[4], out + 2 * i);
        else
            gb::bracket_entry<false>(v[0], v[1], v[2], v[3], v[4], out + 2 * i);
    }
}

}

extern "C" {

// the device sampler ghost_bor_sample_ibc on the host: out[i][j][l] complex
// (interleaved), the same loop body with libm's sqrt / sin / cos
void host_sample_ibc(int nr, int np_, int nxi, const double *rho_p, const double *z_p,
                     const double *tr_p, const double *tz_p, const double *rho_q, const double *z_q,
                     const double *tr_q, const double *tz_q, double k, const double *cx_tab,
                     const double *sx_tab, double *o_tt, double *o_tf, double *o_ft, double *o_ff)
{
    double *outs[4] = {o_tt, o_tf, o_ft, o_ff};
    for (int i = 0; i < nr; ++i)
        for (int j = 0; j < np_; ++j) {
            const double Rz = z_p[i] - z_q[j], rp = rho_p[i], rq = rho_q[j];
            for (int l = 0; l < nxi; ++l) {
                const double cx = cx_tab[l], sx = sx_tab[l];
                const double Rx = rp - rq * cx, Ry = rq * sx;
                double R = std::sqrt(Rx * Rx + Ry * Ry + Rz * Rz);
                if (R < 1e-30) R = 1e-30;
                const double amp = 1.0 / (4.0 * 3.14159265358979323846 * R * R * R);
                const double kr = k * R, sn = std::sin(kr), cs = std::cos(kr);
                const double pr = amp * (cs + kr * sn), pim = amp * (kr * cs - sn);
                double f[4];
                gb::ibc_sample_factors(rp, rq, Rz, tr_p[i], tz_p[i], tr_q[j], tz_q[j], cx, sx, f);
                const size_t o = 2 * (((size_t)i * np_ + j) * nxi + l);
                for (int u = 0; u < 4; ++u) {
                    outs[u][o] = f[u] * pr;
                    outs[u][o + 1] = f[u] * pim;
                }
            }
        }
}

}

#include "medium.cuh"

extern "C" {

// in [n][3] = (R, k_r, k_i); out [n][6] = g (re, im), p (re, im), 1/k^2 (re, im)
void host_complex_k(int n, const double *in, double *out)
{
    for (int i = 0; i < n; ++i) {
        const double *v = in + 3 * i;
        gb::ck_green(v[0], v[1], v[2], 1.0, out + 6 * i);
        gb::ck_bracket(v[0], v[1], v[2], 1.0, out + 6 * i + 2);
        gb::ck_inv_k2(v[1], v[2], out + 6 * i + 4);
    }
}

}
