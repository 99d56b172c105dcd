// capi.cu -- library-level entry points: version, error text, and the
// drop-in device samplers with the reference's ctypes argument meaning
// (bor_stream_kernel.c:26-48 sample_g, :51-106 sample_mfie, :108-150
// sample_ibc).
#include "common.cuh"
#include "brackets.cuh"

#include <stdio.h>
#include <string.h>

namespace gb {

static thread_local char g_last_error[256] = "";
static unsigned long long g_launches = 0;

void set_last_error(const char *msg)
{
    strncpy(g_last_error, msg, sizeof(g_last_error) - 1);
    g_last_error[sizeof(g_last_error) - 1] = 0;
}

int check_launch(const char *where)
{
    __atomic_add_fetch(&g_launches, 1ULL, __ATOMIC_RELAXED);
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return GHOST_BOR_OK;
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", where, cudaGetErrorString(e));
    set_last_error(buf);
    return GHOST_BOR_ECUDA;
}

namespace {

constexpr double R_MIN = 1e-30;   // coincident-point clamp of the reference sampler

// out[i][j][l] for one (i, j) pair per block row, l over threads
__global__ void sample_g_kernel(int nr, int np_, int nxi, const double *__restrict__ rho_p,
                                const double *__restrict__ z_p, const double *__restrict__ rho_q,
                                const double *__restrict__ z_q, double k,
                                const double *__restrict__ sin2, double2 *__restrict__ out)
{
    const long long pair = blockIdx.y * (long long)gridDim.z + blockIdx.z;
    if (pair >= (long long)nr * np_) return;
    const int i = (int)(pair / np_), j = (int)(pair % np_);
    const double dr = rho_p[i] - rho_q[j], dz = z_p[i] - z_q[j];
    const double d2 = dr * dr + dz * dz, rr4 = 4.0 * rho_p[i] * rho_q[j];
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nxi; l += gridDim.x * blockDim.x) {
        double R = sqrt(d2 + rr4 * sin2[l]);
        if (R < R_MIN) R = R_MIN;
        const double amp = 1.0 / (4.0 * GB_PI * R);
        double s, c;
        sincos(k * R, &s, &c);
        out[pair * nxi + l] = make_double2(amp * c, -amp * s);
    }
}

__global__ void sample_mfie_kernel(int nr, int np_, int nxi,
                                   const double *__restrict__ rho_p, const double *__restrict__ z_p,
                                   const double *__restrict__ tr_p, const double *__restrict__ tz_p,
                                   const double *__restrict__ rho_q, const double *__restrict__ z_q,
                                   const double *__restrict__ tr_q, const double *__restrict__ tz_q,
                                   double k, const double *__restrict__ cx_tab, const double *__restrict__ sx_tab,
                                   double2 *__restrict__ o_tt, double2 *__restrict__ o_tf,
                                   double2 *__restrict__ o_ft, double2 *__restrict__ o_ff)
{
    const long long pair = blockIdx.y * (long long)gridDim.z + blockIdx.z;
    if (pair >= (long long)nr * np_) return;
    const int i = (int)(pair / np_), j = (int)(pair % np_);
    const double Rz = z_p[i] - z_q[j];
    const double trp = tr_p[i], tzp = tz_p[i], trq = tr_q[j], tzq = tz_q[j];
    const double rp = rho_p[i], rq = rho_q[j];
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nxi; l += gridDim.x * blockDim.x) {
        const double cx = cx_tab[l], sx = sx_tab[l];
        const double Rx = rp - rq * cx, Ry = rq * sx;
        double R = sqrt(Rx * Rx + Ry * Ry + Rz * Rz);
        if (R < R_MIN) R = R_MIN;
        const double amp = 1.0 / (4.0 * GB_PI * R * R * R);
        const double kr = k * R;
        double sn, cs;
        sincos(kr, &sn, &cs);
        const double pr = amp * (cs + kr * sn), pim = amp * (kr * cs - sn);
        const double WtR = trp * Rx + tzp * Rz, WfR = Ry, nR = -tzp * Rx + trp * Rz;
        const double n_tq = -tzp * trq * cx + trp * tzq, n_fq = -tzp * sx;
        const double Wt_tq = trp * trq * cx + tzp * tzq, Wt_fq = trp * sx;
        const double Wf_tq = -trq * sx, Wf_fq = cx;
        const long long o = pair * nxi + l;
        double f;
        f = -(WtR * n_tq - Wt_tq * nR); o_tt[o] = make_double2(f * pr, f * pim);
        f = -(WtR * n_fq - Wt_fq * nR); o_tf[o] = make_double2(f * pr, f * pim);
        f = -(WfR * n_tq - Wf_tq * nR); o_ft[o] = make_double2(f * pr, f * pim);
        f = -(WfR * n_fq - Wf_fq * nR); o_ff[o] = make_double2(f * pr, f * pim);
    }
}

__global__ void sample_ibc_kernel(int nr, int np_, int nxi,
                                  const double *__restrict__ rho_p, const double *__restrict__ z_p,
                                  const double *__restrict__ tr_p, const double *__restrict__ tz_p,
                                  const double *__restrict__ rho_q, const double *__restrict__ z_q,
                                  const double *__restrict__ tr_q, const double *__restrict__ tz_q,
                                  double k, const double *__restrict__ cx_tab, const double *__restrict__ sx_tab,
                                  double2 *__restrict__ o_tt, double2 *__restrict__ o_tf,
                                  double2 *__restrict__ o_ft, double2 *__restrict__ o_ff)
{
    const long long pair = blockIdx.y * (long long)gridDim.z + blockIdx.z;
    if (pair >= (long long)nr * np_) return;
    const int i = (int)(pair / np_), j = (int)(pair % np_);
    const double Rz = z_p[i] - z_q[j];
    const double rp = rho_p[i], rq = rho_q[j];
    for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < nxi; l += gridDim.x * blockDim.x) {
        const double cx = cx_tab[l], sx = sx_tab[l];
        const double Rx = rp - rq * cx, Ry = rq * sx;
        double R = sqrt(Rx * Rx + Ry * Ry + Rz * Rz);
        if (R < R_MIN) R = R_MIN;
        const double amp = 1.0 / (4.0 * GB_PI * R * R * R);
        const double kr = k * R;
        double sn, cs;
        sincos(kr, &sn, &cs);
        const double pr = amp * (cs + kr * sn), pim = amp * (kr * cs - sn);
        double f[4];
        ibc_sample_factors(rp, rq, Rz, tr_p[i], tz_p[i], tr_q[j], tz_q[j], cx, sx, f);
        const long long o = pair * nxi + l;
        o_tt[o] = make_double2(f[0] * pr, f[0] * pim);
        o_tf[o] = make_double2(f[1] * pr, f[1] * pim);
        o_ft[o] = make_double2(f[2] * pr, f[2] * pim);
        o_ff[o] = make_double2(f[3] * pr, f[3] * pim);
    }
}

dim3 pair_grid(int nr, int np_, int nxi)
{
    const long long pairs = (long long)nr * np_;
    const unsigned gz = (unsigned)(pairs < 65535 ? pairs : 65535);
    const unsigned gy = (unsigned)((pairs + gz - 1) / gz);
    const unsigned gx = (unsigned)((nxi + 127) / 128 < 4 ? (nxi + 127) / 128 : 4);
    return dim3(gx, gy, gz);
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" int ghost_bor_version(void) { return 100; }

extern "C" const char *ghost_bor_last_error(void) { return g_last_error; }

extern "C" long long ghost_bor_launch_count(void)
{
    return (long long)__atomic_load_n(&g_launches, __ATOMIC_RELAXED);
}

extern "C" int ghost_bor_sample_g(int nr, int np_, int nxi,
                                  const double *rho_p, const double *z_p,
                                  const double *rho_q, const double *z_q,
                                  double k, const double *sin2_tab, double *out, void *stream)
{
    if (nr < 0 || np_ < 0 || nxi < 1 || (nr > 0 && np_ > 0 && (!rho_p || !z_p || !rho_q || !z_q || !sin2_tab || !out)))
        return GHOST_BOR_EINVAL;
    if ((long long)nr * np_ == 0) return GHOST_BOR_OK;
    if ((long long)nr * np_ > 65535LL * 65535LL) return GHOST_BOR_EINVAL;
    sample_g_kernel<<<pair_grid(nr, np_, nxi), 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        nr, np_, nxi, rho_p, z_p, rho_q, z_q, k, sin2_tab, reinterpret_cast<double2 *>(out));
    return check_launch("sample_g");
}

extern "C" int ghost_bor_sample_mfie(int nr, int np_, int nxi,
                                     const double *rho_p, const double *z_p,
                                     const double *tr_p, const double *tz_p,
                                     const double *rho_q, const double *z_q,
                                     const double *tr_q, const double *tz_q,
                                     double k, const double *cos_tab, const double *sin_tab,
                                     double *o_tt, double *o_tf, double *o_ft, double *o_ff, void *stream)
{
    if (nr < 0 || np_ < 0 || nxi < 1) return GHOST_BOR_EINVAL;
    if ((long long)nr * np_ == 0) return GHOST_BOR_OK;
    if (!rho_p || !z_p || !tr_p || !tz_p || !rho_q || !z_q || !tr_q || !tz_q || !cos_tab || !sin_tab ||
        !o_tt || !o_tf || !o_ft || !o_ff || (long long)nr * np_ > 65535LL * 65535LL)
        return GHOST_BOR_EINVAL;
    sample_mfie_kernel<<<pair_grid(nr, np_, nxi), 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        nr, np_, nxi, rho_p, z_p, tr_p, tz_p, rho_q, z_q, tr_q, tz_q, k, cos_tab, sin_tab,
        reinterpret_cast<double2 *>(o_tt), reinterpret_cast<double2 *>(o_tf),
        reinterpret_cast<double2 *>(o_ft), reinterpret_cast<double2 *>(o_ff));
    return check_launch("sample_mfie");
}

extern "C" int ghost_bor_sample_ibc(int nr, int np_, int nxi,
                                    const double *rho_p, const double *z_p,
                                    const double *tr_p, const double *tz_p,
                                    const double *rho_q, const double *z_q,
                                    const double *tr_q, const double *tz_q,
                                    double k, const double *cos_tab, const double *sin_tab,
                                    double *o_tt, double *o_tf, double *o_ft, double *o_ff, void *stream)
{
    if (nr < 0 || np_ < 0 || nxi < 1) return GHOST_BOR_EINVAL;
    if ((long long)nr * np_ == 0) return GHOST_BOR_OK;
    if (!rho_p || !z_p || !tr_p || !tz_p || !rho_q || !z_q || !tr_q || !tz_q || !cos_tab || !sin_tab ||
        !o_tt || !o_tf || !o_ft || !o_ff || (long long)nr * np_ > 65535LL * 65535LL)
        return GHOST_BOR_EINVAL;
    sample_ibc_kernel<<<pair_grid(nr, np_, nxi), 128, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
        nr, np_, nxi, rho_p, z_p, tr_p, tz_p, rho_q, z_q, tr_q, tz_q, k, cos_tab, sin_tab,
        reinterpret_cast<double2 *>(o_tt), reinterpret_cast<double2 *>(o_tf),
        reinterpret_cast<double2 *>(o_ft), reinterpret_cast<double2 *>(o_ff));
    return check_launch("sample_ibc");
}
