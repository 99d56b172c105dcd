// Host build of the bracket-fill coefficient code (csrc/brackets.cuh) for the
// CPU tests: the same expressions the MFIE and IBC fill kernels compile.
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
