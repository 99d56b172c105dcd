// rhs.cu -- plane-wave excitation for every (mode, angle, polarisation) and
// the far-field mode sum by reciprocity.
//
// Replaces rhs_mode (bor_solver.py:625-645), rhs_mfie_mode (:437-461) and
// farfield_mode (:659-708).  The reference evaluates scipy jv three times per
// Gauss point per column; here one thread per (point, angle) builds the whole
// table J_0..J_{M+1}(k rho sin theta) by J. C. P. Miller's backward recurrence
// J_{n-1} = (2n/x) J_n - J_{n+1}, normalised with J_0 + 2 sum_k J_2k = 1
// (Abramowitz & Stegun 9.1.27 / 9.1.46, the standard published method), FP64.
//
// Far field: the reference projects every solution column on the same Bessel
// integrands as the excitation, so F_theta = c (D V_VV)^T x and
// F_phi = -c (D V_HH)^T x with c = -j k eta0 / (4 pi), D = diag(I, -I): a
// batched dot product of each solution column with its own excitation.
#include "common.cuh"

namespace gb {
namespace {

constexpr int MAX_ORD = 512;      // J_n table held per thread (orders 0..M+1)
constexpr int kMaxGridY = 65535;  // grid y limit: points and nodes stride over it
constexpr double ETA0 = 376.730313668;

// Bessel J_0..J_nmax(x), x >= 0, into out[0..nmax] (strided).
__device__ void bessel_table(double x, int nmax, double *__restrict__ out, long long stride)
{
    if (x == 0.0) {
        out[0] = 1.0;
        for (int n = 1; n <= nmax; ++n) out[n * stride] = 0.0;
        return;
    }
    double loc[MAX_ORD];
    const double K = fmax((double)nmax, ceil(x)) + 1.0;
    int nst = 2 * (((int)K + (int)sqrt(160.0 * K)) / 2);     // even start, far above max(n, x)
    double jp1 = 0.0, jn = 1e-30, sum = 0.0;
    const double tx = 2.0 / x;
    for (int n = nst; n >= 1; --n) {
        const double jm1 = n * tx * jn - jp1;             // J_{n-1}
        jp1 = jn;
        jn = jm1;
        if (n - 1 <= nmax) loc[n - 1] = jn;
        if (((n - 1) & 1) == 0 && n - 1 > 0) sum += 2.0 * jn;
        if (fabs(jn) > 1e250) {                            // rescale everything kept so far
            jn *= 1e-250; jp1 *= 1e-250; sum *= 1e-250;
            for (int i = n - 1; i <= nmax; ++i) loc[i] *= 1e-250;
        }
    }
    // also fix the n = nmax+1..nst values we did not keep (not needed)
    sum += jn;                                             // J_0 term
    const double inv = 1.0 / sum;
    for (int n = 0; n <= nmax; ++n) out[n * stride] = loc[n] * inv;
}

// Jtab[(p * Mp + n) * T + it], Ph[p * T + it] = exp(j k cos(theta) z_p)
__global__ void bessel_phase_kernel(int P, int Mp, int T, double k, const double *__restrict__ geo,
                                    const double *__restrict__ thetas, double *__restrict__ Jtab,
                                    double2 *__restrict__ Ph)
{
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= T) return;
    const double th = thetas[it] * (GB_PI / 180.0);
    double st, ct;
    sincos(th, &st, &ct);
    // Gauss points stride over grid y (at most 65535 blocks in y)
    for (int p = blockIdx.y; p < P; p += gridDim.y) {
        const double rho = geo[p], z = geo[P + p];
        bessel_table(k * rho * st, Mp - 1, Jtab + (size_t)p * Mp * T + it, T);
        double s, c;
        sincos(k * ct * z, &s, &c);
        Ph[(size_t)p * T + it] = make_double2(c, s);
    }
}

__device__ __forceinline__ double2 ipow_times(int n, double v)
{
    // i^n * v for n >= 0
    switch (n & 3) {
        case 0: return make_double2(v, 0.0);
        case 1: return make_double2(0.0, v);
        case 2: return make_double2(-v, 0.0);
        default: return make_double2(0.0, -v);
    }
}

// B[m][row][2 it + pol]: one thread per (it), nodes striding over grid y, blockIdx.z = m
__global__ void rhs_kernel(int N, int Nn, int Mp, int T, double k, double ce, double ch,
                           const double2 *__restrict__ hw,
                           const double *__restrict__ geo, const double *__restrict__ thetas,
                           const double *__restrict__ Jtab, const double2 *__restrict__ Ph,
                           const int *__restrict__ mask_rows, double2 *__restrict__ B,
                           long long ldb, long long mode_stride)
{
    const int it = blockIdx.x * blockDim.x + threadIdx.x;
    const int m = blockIdx.z;
    if (it >= T) return;
    const int P = 4 * N;
    const double th = thetas[it] * (GB_PI / 180.0);
    double st, ct;
    sincos(th, &st, &ct);
    for (int i = blockIdx.y; i < Nn; i += gridDim.y) {
    double2 vt[2] = {make_double2(0, 0), make_double2(0, 0)};   // [pol]
    double2 vf[2] = {make_double2(0, 0), make_double2(0, 0)};
    const int nlo = abs(m - 1), nhi = m + 1;
    for (int side = 0; side < 2; ++side) {
        const int el = (side == 0) ? i - 1 : i;      // element with node i as its end 1 / end 0
        if (el < 0 || el >= N) continue;
        for (int g = 0; g < 4; ++g) {
            const int p = 4 * el + g;
            // T_i(p) w rho: node i is end 1 of element i-1 (side 0) and end 0 of element i
            const double cw = (side == 0) ? geo[(size_t)4 * P + p] : geo[(size_t)3 * P + p];
            const double tr = geo[(size_t)9 * P + p], tz = geo[(size_t)10 * P + p];
            const double *J = Jtab + (size_t)p * Mp * T + it;
            const double2 jl = ipow_times(nlo, J[(size_t)nlo * T]);
            const double2 jh = ipow_times(nhi, J[(size_t)nhi * T]);
            const double2 j0 = ipow_times(m, J[(size_t)m * T]);
            const double2 Ic = make_double2(GB_PI * (jl.x + jh.x), GB_PI * (jl.y + jh.y));
            // Is = (pi / j) (jl - jh) = -j pi (jl - jh)
            const double2 Is = make_double2(GB_PI * (jl.y - jh.y), -GB_PI * (jl.x - jh.x));
            const double2 I1 = make_double2(2.0 * GB_PI * j0.x, 2.0 * GB_PI * j0.y);
            const double2 ph = Ph[(size_t)p * T + it];
            const double2 com = make_double2(cw * ph.x, cw * ph.y);
            // EFIE parts
            double2 etv = make_double2(ct * tr * Ic.x - st * tz * I1.x, ct * tr * Ic.y - st * tz * I1.y);
            double2 efv = make_double2(-ct * Is.x, -ct * Is.y);
            double2 eth = make_double2(tr * Is.x, tr * Is.y);
            double2 efh = Ic;
            double2 tv = make_double2(ce * etv.x, ce * etv.y), fv = make_double2(ce * efv.x, ce * efv.y);
            double2 thh = make_double2(ce * eth.x, ce * eth.y), fh = make_double2(ce * efh.x, ce * efh.y);
            if (hw) {
                // n x H parts with the complex weight of the element (Z_s for the
                // far field of an impedance surface): c2 = ch w(el) / eta0
                const double2 w = hw[el];
                const double2 c2 = make_double2(ch / ETA0 * w.x, ch / ETA0 * w.y);
                const double2 a = cmul(c2, Ic), b = cmul(c2, Is);
                const double2 h = cmul(c2, make_double2(ct * tr * Ic.x - st * tz * I1.x,
                                                        ct * tr * Ic.y - st * tz * I1.y));
                tv.x += a.x; tv.y += a.y;
                fv.x -= tr * b.x; fv.y -= tr * b.y;
                thh.x += ct * b.x; thh.y += ct * b.y;
                fh.x += h.x; fh.y += h.y;
            } else if (ch != 0.0) {
                const double c2 = ch / ETA0;
                // MFIE parts: VV et = Ic, ef = -t_rho Is ; HH et = ct Is, ef = ct t_rho Ic - st t_z I1
                tv.x += c2 * Ic.x; tv.y += c2 * Ic.y;
                fv.x -= c2 * tr * Is.x; fv.y -= c2 * tr * Is.y;
                thh.x += c2 * ct * Is.x; thh.y += c2 * ct * Is.y;
                fh.x += c2 * (ct * tr * Ic.x - st * tz * I1.x);
                fh.y += c2 * (ct * tr * Ic.y - st * tz * I1.y);
            }
            vt[0] = cfma(com, tv, vt[0]);
            vf[0] = cfma(com, fv, vf[0]);
            vt[1] = cfma(com, thh, vt[1]);
            vf[1] = cfma(com, fh, vf[1]);
        }
    }
    const int *mr = mask_rows + 4 * m;
    const bool mt = (mr[0] == i || mr[1] == i || mr[2] == i || mr[3] == i);
    const bool mf = (mr[0] == Nn + i || mr[1] == Nn + i || mr[2] == Nn + i || mr[3] == Nn + i);
    double2 *Bm = B + (size_t)m * mode_stride;
    const double2 z = make_double2(0.0, 0.0);
    Bm[(size_t)i * ldb + 2 * it + 0] = mt ? z : vt[0];
    Bm[(size_t)i * ldb + 2 * it + 1] = mt ? z : vt[1];
    Bm[(size_t)(Nn + i) * ldb + 2 * it + 0] = mf ? z : vf[0];
    Bm[(size_t)(Nn + i) * ldb + 2 * it + 1] = mf ? z : vf[1];
    }
}

template <class R>
__global__ void farfield_kernel(int n, int nrhs, int Nn, int rows_per_block, double pref_im,
                                const double *__restrict__ mode_weight,
                                const double2 *__restrict__ Ve, long long ldv, long long sv,
                                const C<R> *__restrict__ X, long long ldx, long long sx,
                                double2 *__restrict__ dF)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.z;
    if (c >= nrhs) return;
    const int r0 = blockIdx.y * rows_per_block;
    const int r1 = min(n, r0 + rows_per_block);
    const double2 *V = Ve + (size_t)b * sv;
    const C<R> *Xb = X + (size_t)b * sx;
    double ax = 0.0, ay = 0.0;
    for (int r = r0; r < r1; ++r) {
        const double2 v = V[(size_t)r * ldv + c];
        const C<R> xr = Xb[(size_t)r * ldx + c];
        const double xx = (double)xr.x, xy = (double)xr.y;
        const double sgn = (r < Nn) ? 1.0 : -1.0;
        ax += sgn * (v.x * xx - v.y * xy);
        ay += sgn * (v.x * xy + v.y * xx);
    }
    // pref = -j k eta0/(4 pi) = j * pref_im with pref_im < 0 ; times weight and pol sign
    const double wgt = mode_weight[b] * ((c & 1) ? -1.0 : 1.0);
    const double2 out = make_double2(-pref_im * ay * wgt, pref_im * ax * wgt);
    atomicAdd(&dF[(size_t)b * nrhs + c].x, out.x);
    atomicAdd(&dF[(size_t)b * nrhs + c].y, out.y);
}

}  // namespace
}  // namespace gb

extern "C" long long ghost_bor_rhs_workspace(int n_elem, int m_max, int n_theta)
{
    const long long P = 4LL * n_elem;
    return P * (m_max + 2) * n_theta * 8 + P * n_theta * 16 + 256;
}

namespace gb {
namespace {

int rhs_launch(int n_elem, int m_max, int n_theta, double k, double coef_e, double coef_h,
               const double *h_weight, const double *geo, const double *thetas_deg,
               const int *mask_rows, double *B, long long ldb, long long mode_stride,
               void *work, void *stream)
{
    const int Mp = m_max + 2;
    if (n_elem < 1 || m_max < 0 || Mp > MAX_ORD || n_theta < 1 || !geo || !thetas_deg || !mask_rows ||
        !B || !work || ldb < 2LL * n_theta || mode_stride < ldb * 2LL * (n_elem + 1))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int P = 4 * n_elem;
    double *Jtab = reinterpret_cast<double *>(work);
    double2 *Ph = reinterpret_cast<double2 *>(
        (reinterpret_cast<uintptr_t>(Jtab + (size_t)P * Mp * n_theta) + 15) & ~uintptr_t(15));
    dim3 g1((n_theta + 63) / 64, P < kMaxGridY ? P : kMaxGridY);
    bessel_phase_kernel<<<g1, 64, 0, st>>>(P, Mp, n_theta, k, geo, thetas_deg, Jtab, Ph);
    int rc = check_launch("rhs: bessel");
    if (rc) return rc;
    dim3 g2((n_theta + 63) / 64, n_elem + 1 < kMaxGridY ? n_elem + 1 : kMaxGridY, m_max + 1);
    rhs_kernel<<<g2, 64, 0, st>>>(n_elem, n_elem + 1, Mp, n_theta, k, coef_e, coef_h,
                                  reinterpret_cast<const double2 *>(h_weight), geo, thetas_deg,
                                  Jtab, Ph, mask_rows, reinterpret_cast<double2 *>(B), ldb, mode_stride);
    return check_launch("rhs");
}

}  // namespace
}  // namespace gb

extern "C" int ghost_bor_rhs(int n_elem, int m_max, int n_theta, double k,
                             double coef_e, double coef_h,
                             const double *geo, const double *thetas_deg,
                             const int *mask_rows, double *B, long long ldb, long long mode_stride,
                             void *work, void *stream)
{
    return gb::rhs_launch(n_elem, m_max, n_theta, k, coef_e, coef_h, nullptr, geo, thetas_deg, mask_rows, B,
                          ldb, mode_stride, work, stream);
}

extern "C" int ghost_bor_rhs_weighted(int n_elem, int m_max, int n_theta, double k,
                                      double coef_e, double coef_h, const double *h_weight,
                                      const double *geo, const double *thetas_deg,
                                      const int *mask_rows, double *B, long long ldb, long long mode_stride,
                                      void *work, void *stream)
{
    if (!h_weight) return GHOST_BOR_EINVAL;
    return gb::rhs_launch(n_elem, m_max, n_theta, k, coef_e, coef_h, h_weight, geo, thetas_deg, mask_rows, B,
                          ldb, mode_stride, work, stream);
}

extern "C" int ghost_bor_farfield(int prec, int batch, int n, int nrhs, int Nn, double k,
                                  const double *mode_weight,
                                  const double *Ve, long long ldv, long long stride_v,
                                  const void *X, long long ldx, long long stride_x,
                                  double *dF, void *stream)
{
    using namespace gb;
    if (batch < 1 || n < 1 || nrhs < 1 || !mode_weight || !Ve || !X || !dF || ldv < nrhs || ldx < nrhs)
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int rpb = 256;
    dim3 grid((nrhs + 127) / 128, (n + rpb - 1) / rpb, batch);
    const double pref_im = -k * 376.730313668 / (4.0 * GB_PI);
    if (cudaMemsetAsync(dF, 0, sizeof(double) * 2 * (size_t)batch * nrhs, st) != cudaSuccess)
        return check_launch("farfield: memset");
    if (prec == GHOST_BOR_F64)
        farfield_kernel<double><<<grid, 128, 0, st>>>(n, nrhs, Nn, rpb, pref_im, mode_weight,
            reinterpret_cast<const double2 *>(Ve), ldv, stride_v,
            reinterpret_cast<const double2 *>(X), ldx, stride_x, reinterpret_cast<double2 *>(dF));
    else if (prec == GHOST_BOR_F32)
        farfield_kernel<float><<<grid, 128, 0, st>>>(n, nrhs, Nn, rpb, pref_im, mode_weight,
            reinterpret_cast<const double2 *>(Ve), ldv, stride_v,
            reinterpret_cast<const float2 *>(X), ldx, stride_x, reinterpret_cast<double2 *>(dF));
    else
        return GHOST_BOR_EINVAL;
    return check_launch("farfield");
}

// ---------------------------------------------------------------------------
// Allocation-free excitation.
//
// Some callers cannot allocate device memory while they solve: a service that
// reserves all GPU memory for its own arena at start-up, or a host thread that
// must not call cudaMalloc/cudaFree because those calls can synchronise the
// whole device and fail once memory is fragmented.  For them the Bessel /
// phase workspace of ghost_bor_rhs lives in one file-scope device array of
// fixed size that every GPU loading this library keeps until the process
// exits; the sweep is processed in blocks of angles that fit in it.
//
// Limits and rules: one angle needs 4*n_elem*((m_max+2)*8 + 16) bytes of the
// array; larger problems are rejected.  The array is shared by every call and
// keeps the previous call's contents (everything read is written first in the
// same call, so nothing needs clearing); calls that overlap on the GPU (other
// streams, other host threads) race on it and must be serialised by the
// caller.  The first call on each device looks up the array's device address
// with cudaGetSymbolAddress while that device is current; make that first call
// before any stream capture.  The address is cached per device ordinal for the
// life of the process: after cudaDeviceReset it is stale, so a process that
// resets a device must not call this entry point on it again.
// ---------------------------------------------------------------------------
namespace gb {
namespace {

constexpr long long kRhsScratchBytes = 64LL << 20;
__device__ __align__(256) unsigned char g_rhs_scratch[kRhsScratchBytes];

constexpr int kMaxDevices = 64;
void *g_rhs_scratch_ptr[kMaxDevices] = {};

void *rhs_scratch_for_current_device()
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    void *p = __atomic_load_n(&g_rhs_scratch_ptr[dev], __ATOMIC_ACQUIRE);
    if (p) return p;
    if (cudaGetSymbolAddress(&p, g_rhs_scratch) != cudaSuccess || !p) return nullptr;
    __atomic_store_n(&g_rhs_scratch_ptr[dev], p, __ATOMIC_RELEASE);
    return p;
}

}  // namespace
}  // namespace gb

extern "C" long long ghost_bor_rhs_noalloc_capacity(void) { return gb::kRhsScratchBytes; }

extern "C" int ghost_bor_rhs_noalloc(int n_elem, int m_max, int n_theta, double k,
                                     double coef_e, double coef_h,
                                     const double *geo, const double *thetas_deg,
                                     const int *mask_rows, double *B, long long ldb, long long mode_stride,
                                     void *stream)
{
    using namespace gb;
    const int Mp = m_max + 2;
    if (n_elem < 1 || m_max < 0 || Mp > MAX_ORD || n_theta < 1 || !geo || !thetas_deg || !mask_rows ||
        !B || ldb < 2LL * n_theta || mode_stride < ldb * 2LL * (n_elem + 1))
        return GHOST_BOR_EINVAL;
    const long long P = 4LL * n_elem;
    const long long per_angle = P * Mp * 8 + P * 16;
    const long long usable = kRhsScratchBytes - 256;          // alignment slack for the phase table
    if (per_angle > usable) {
        set_last_error("ghost_bor_rhs_noalloc: one angle needs more than the 64 MiB static workspace "
                       "(4*n_elem*((m_max+2)*8+16) bytes); use ghost_bor_rhs with a caller workspace");
        return GHOST_BOR_EINVAL;
    }
    void *scratch = rhs_scratch_for_current_device();
    if (!scratch) {
        set_last_error("ghost_bor_rhs_noalloc: cudaGetSymbolAddress of the static workspace failed");
        return GHOST_BOR_ECUDA;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int chunk = (int)(usable / per_angle < n_theta ? usable / per_angle : n_theta);
    for (int it0 = 0; it0 < n_theta; it0 += chunk) {
        const int T = (n_theta - it0 < chunk) ? n_theta - it0 : chunk;
        double *Jtab = reinterpret_cast<double *>(scratch);
        double2 *Ph = reinterpret_cast<double2 *>(
            (reinterpret_cast<uintptr_t>(Jtab + (size_t)P * Mp * T) + 15) & ~uintptr_t(15));
        dim3 g1((T + 63) / 64, (unsigned)(P < kMaxGridY ? P : kMaxGridY));
        bessel_phase_kernel<<<g1, 64, 0, st>>>((int)P, Mp, T, k, geo, thetas_deg + it0, Jtab, Ph);
        int rc = check_launch("rhs_noalloc: bessel");
        if (rc) return rc;
        dim3 g2((T + 63) / 64, n_elem + 1 < kMaxGridY ? n_elem + 1 : kMaxGridY, m_max + 1);
        rhs_kernel<<<g2, 64, 0, st>>>(n_elem, n_elem + 1, Mp, T, k, coef_e, coef_h, nullptr, geo,
                                      thetas_deg + it0,
                                      Jtab, Ph, mask_rows, reinterpret_cast<double2 *>(B) + 2 * (size_t)it0,
                                      ldb, mode_stride);
        if ((rc = check_launch("rhs_noalloc"))) return rc;
    }
    return GHOST_BOR_OK;
}
