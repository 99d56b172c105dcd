// mfie_fill.cu -- MFIE operator fill for all azimuthal modes m = 0..M.
//
// Z_MFIE(m) = M/2 - K(m) (bor_solver.py:399-435): K holds the four bracket
// blocks tt, tf, ft, ff of the n x grad G' kernel, M is the mass matrix
// 2 pi B_T diag(w rho) B_T^T (bor_solver.py:389-397).  Replaces the
// reference's bracket sampler (bor_stream_kernel.c:65-106, bor_kernels.py:
// 273-306) with its FFT and contraction (bor_streaming.py:241-246, 378-385)
// for the far pairs |e - f| >= 2, and the near bracket path
// (bor_kernels.py:334-431, bor_solver.py:372-387, 415-426) for |e - f| <= 1.
//
// Bracket algebra.  With the test point at phi = 0, the source at
// phi' = -xi, d = (rho - rho', z - z'), s2 = sin^2(xi/2) and unit tangents
// t = (t_rho, t_z), t' the reference's four brackets
//   F_tt = -p (WtR n_tq - Wt_tq nR),   F_tf = -p (WtR n_fq - Wt_fq nR),
//   F_ft = -p (Ry n_tq - Wf_tq nR),    F_ff = -p (Ry n_fq - Wf_fq nR)
// reduce exactly (the s2^2 terms and, in F_ft, the s2 terms cancel) to
//   F_tt = -p (c0 + c1 s2)             c0 = d x t'  = d_rho t'_z - d_z t'_rho
//   F_ff =  p (N0 - 2 s2 (N0 - rho' t_z))
//   F_tf =  p sin(xi) d_z
//   F_ft = -p sin(xi) e0
// with N0 = t x d, X0 = t x t', A0 = t . d, D0 = t . t',
// c1 = 2 (A0 t_z t'_rho + t_rho rho' X0 + D0 t_z rho' + t_rho t'_rho N0),
// e0 = rho' X0 + t'_rho N0.  So three azimuth transforms of p -- C[p],
// C[p s2] (cosine) and S[p sin xi] (sine) -- give all four brackets, and the
// per-sample products of the reference, which cancel for nearby points, are
// never formed.  The combinations c0 C[p] + c1 C[p s2] lose at most a
// factor ~2 to cancellation.
//
// Surface impedance (IBC-EFIE).  The reference's extra operator
// Z_s (M/2) + B (bor_solver.py:499-552: the Z_s-weighted mass term plus the
// rotated principal-value brackets with Z_s at the source, far part from
// bor_kernels.py:449-511 / bor_stream_kernel.c:108-150, near part from
// bor_kernels.py:514-560 on the same graded cells) is the same three
// transforms with another coefficient set (brackets.cuh), the opposite sign
// of the bracket term and a complex weight per source element: the IBC
// instantiations of both kernels below.
#include <type_traits>

#include "common.cuh"
#include "samplers.cuh"
#include "brackets.cuh"

namespace gb {
namespace {

// ---------------------------------------------------------------------------
// far pairs
// ---------------------------------------------------------------------------
constexpr int MEPB = 2;                 // element pairs per CTA
constexpr int MPPB = MEPB * 16;         // Gauss-point pairs per CTA
constexpr int MOG = 8;                  // order groups
constexpr int MNT = 8;                  // orders per thread
constexpr int MTPB = MPPB * MOG;        // 256 threads
constexpr int MNOB = MOG * MNT;         // 64 orders per launch row
constexpr int MJC = 32;                 // azimuth samples per smem chunk

template <class R> struct MfieSmem {
    // phase 1 (transforms):  gsm [MJC][MPPB] C<R>, tabs [MJC][3][MNOB] R, s2s [MJC] S2
    // phase 2 (contraction): Ts [MEPB][MNOB][3][16] C<R>   (aliases phase 1)
    // always:  coef [MEPB][16][6] double, lw [MEPB + 1][2][4] double
    static constexpr size_t p1() {
        return sizeof(C<R>) * MJC * MPPB + sizeof(R) * MJC * 3 * MNOB +
               sizeof(typename BracketSampler<R>::S2) * MJC;
    }
    static constexpr size_t p2() { return sizeof(C<R>) * MEPB * MNOB * 3 * 16; }
    static constexpr size_t head() { return p1() > p2() ? p1() : p2(); }
    static constexpr size_t bytes() {
        return head() + sizeof(double) * (MEPB * 16 * 6 + (MEPB + 1) * 8);
    }
};

// CK: complex wave number k + j ki (FP64 only; a lossy medium's interior)
template <class R, bool IBC, bool CK = false>
__global__ void __launch_bounds__(MTPB)
far_mfie_kernel(int N, int Nn, int M, int h, double k, double sc_re, double sc_im,
                const double *__restrict__ geo, const double *__restrict__ tab,
                const double *__restrict__ sin2, const double2 *__restrict__ wsrc,
                double2 *__restrict__ Z, long long ldz, long long mode_stride, double ki)
{
    static_assert(!CK || sizeof(R) == 8, "complex wave numbers on the FP64 path only");
    using CT = C<R>;
    using Samp = typename std::conditional<CK, BracketSamplerC, BracketSampler<R>>::type;
    using S2 = typename Samp::S2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT *gsm = reinterpret_cast<CT *>(smem_raw);
    R *tabs = reinterpret_cast<R *>(gsm + MJC * MPPB);
    S2 *s2s = reinterpret_cast<S2 *>(tabs + MJC * 3 * MNOB);
    CT *Ts = reinterpret_cast<CT *>(smem_raw);
    double *coef = reinterpret_cast<double *>(smem_raw + MfieSmem<R>::head());
    double *lw = coef + MEPB * 16 * 6;

    const int P = 4 * N;
    const int Mo = M + 1;
    const int fgroups = (N + MEPB - 1) / MEPB;
    const int e = blockIdx.x / fgroups;
    const int f0 = (blockIdx.x % fgroups) * MEPB;
    const int m0 = blockIdx.y * MNOB;
    if (m0 > M) return;
    const int nord = min(MNOB, Mo - m0);

    const int tid = threadIdx.x;
    const int og = tid / MPPB;
    const int pp = tid % MPPB;
    const int ep = pp >> 4, gh = pp & 15;
    const int f = f0 + ep;
    const bool active = (f < N) && (abs(e - f) >= 2);

    // Galerkin weights T w rho of the test element (slot MEPB) and the sources
    for (int i = tid; i < (MEPB + 1) * 8; i += MTPB) {
        const int slot = i / 8, r = i % 8;
        const int el = (slot == MEPB) ? e : min(f0 + slot, N - 1);
        lw[i] = geo[(size_t)(3 + r / 4) * P + 4 * el + (r % 4)];
    }
    for (int i = tid; i < MEPB * 16; i += MTPB) {
        const int el = min(f0 + i / 16, N - 1);
        const int p = 4 * e + ((i & 15) >> 2), q = 4 * el + (i & 3);
        bracket_coefs<IBC>(geo[p], geo[P + p], geo[(size_t)9 * P + p], geo[(size_t)10 * P + p],
                           geo[q], geo[P + q], geo[(size_t)9 * P + q], geo[(size_t)10 * P + q], coef + 6 * i);
    }

    Samp smp;
    {
        const int p = 4 * e + (gh >> 2);
        const int q = 4 * min(f, N - 1) + (gh & 3);
        const double rp = geo[p], zp = geo[P + p];
        const double rq = geo[q], zq = geo[P + q];
        const double dr = rp - rq, dz = zp - zq;
        if constexpr (CK)
            smp.init(dr * dr + dz * dz, 4.0 * rp * rq, k, ki);
        else
            smp.init(dr * dr + dz * dz, 4.0 * rp * rq, k);
    }

    CT acc[3][MNT];
#pragma unroll
    for (int t = 0; t < 3; ++t)
#pragma unroll
        for (int n = 0; n < MNT; ++n) acc[t][n] = mk<R>(R(0), R(0));

    for (int j0 = 0; j0 <= h; j0 += MJC) {
        __syncthreads();
        for (int i = tid; i < MJC * 3 * MNOB; i += MTPB) {
            const int jj = i / (3 * MNOB), t = (i / MNOB) % 3, n = i % MNOB;
            const int j = j0 + jj, m = m0 + n;
            tabs[i] = (j <= h && m < Mo) ? (R)tab[((size_t)t * (h + 1) + j) * Mo + m] : R(0);
        }
        for (int jj = tid; jj < MJC; jj += MTPB) s2s[jj] = Samp::load_s2(sin2, min(j0 + jj, h));
        __syncthreads();
        const int jn = min(MJC, h + 1 - j0);
#pragma unroll 2
        for (int jj = og; jj < MJC; jj += MOG)
            gsm[jj * MPPB + pp] = (active && jj < jn) ? smp(s2s[jj]) : mk<R>(R(0), R(0));
        __syncthreads();
        if (!active) continue;
        for (int jj = 0; jj < jn; ++jj) {
            const CT gv = gsm[jj * MPPB + pp];
#pragma unroll
            for (int t = 0; t < 3; ++t) {
                const R *row = tabs + (jj * 3 + t) * MNOB + og * MNT;
#pragma unroll
                for (int n = 0; n < MNT; ++n) {
                    const R c = row[n];
                    acc[t][n].x = fma(gv.x, c, acc[t][n].x);
                    acc[t][n].y = fma(gv.y, c, acc[t][n].y);
                }
            }
        }
    }
    __syncthreads();                    // phase 1 buffers are reused below
#pragma unroll
    for (int t = 0; t < 3; ++t)
#pragma unroll
        for (int n = 0; n < MNT; ++n)
            Ts[((ep * MNOB + og * MNT + n) * 3 + t) * 16 + gh] = acc[t][n];
    __syncthreads();

    // contraction job (ep, n, ab): the four brackets of order m0 + n between
    // test node e + a and source node f + b, then -scale * K into Z[m]
    for (int job = tid; job < MEPB * nord * 4; job += MTPB) {
        const int jep = job / (nord * 4), n = (job / 4) % nord, ab = job & 3;
        const int a = ab >> 1, b = ab & 1;
        const int ff = f0 + jep;
        if (ff >= N || abs(e - ff) < 2) continue;
        const CT *T = Ts + (jep * MNOB + n) * 3 * 16;
        const double *lt = lw + MEPB * 8 + a * 4;
        const double *ls = lw + jep * 8 + b * 4;
        double2 ktt = make_double2(0, 0), kff = ktt, ktf = ktt, kft = ktt;
#pragma unroll 4
        for (int g2 = 0; g2 < 16; ++g2) {
            const double w = lt[g2 >> 2] * ls[g2 & 3];
            const double *cf = coef + (jep * 16 + g2) * 6;
            const CT cp = T[0 * 16 + g2], cs = T[1 * 16 + g2], sx = T[2 * 16 + g2];
            const double cpx = cp.x, cpy = cp.y, csx = cs.x, csy = cs.y, sxx = sx.x, sxy = sx.y;
            ktt.x += w * (cf[0] * cpx + cf[1] * csx); ktt.y += w * (cf[0] * cpy + cf[1] * csy);
            kff.x += w * (cf[2] * cpx + cf[3] * csx); kff.y += w * (cf[2] * cpy + cf[3] * csy);
            ktf.x += w * cf[4] * sxx; ktf.y += w * cf[4] * sxy;
            kft.x += w * cf[5] * sxx; kft.y += w * cf[5] * sxy;
        }
        // K_tf = -j ktf, K_ft = -j kft; the block value is -scale K (MFIE) or
        // +scale Z_s(f) K (IBC, Z_s of the source element)
        const double2 K[4] = {ktt, make_double2(ktf.y, -ktf.x), make_double2(kft.y, -kft.x), kff};
        double s_re = sc_re, s_im = sc_im;
        if (IBC && wsrc) {
            const double2 w = wsrc[ff];
            s_re = sc_re * w.x - sc_im * w.y;
            s_im = sc_re * w.y + sc_im * w.x;
        }
        double2 *Zm = Z + (size_t)(m0 + n) * mode_stride;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const long long row = e + a + (q >> 1) * Nn, col = ff + b + (q & 1) * Nn;
            double v[2];
            bracket_entry<IBC>(K[q].x, K[q].y, 0.0, s_re, s_im, v);
            catomic_add(Zm + row * ldz + col, make_double2(v[0], v[1]));
        }
    }
}

// ---------------------------------------------------------------------------
// near pairs |e - f| <= 1 (graded cells, sinh core + Gauss tail) and mass.
// Persistent grid; per batch of 128 point pairs each thread evaluates its
// azimuth nodes once (FP64 transcendentals; this kernel is FP64 throughout)
// into a per-CTA scratch, then each
// chunk of NCM orders projects from it (see near_fill.cu).
// ---------------------------------------------------------------------------
constexpr int NTPB = 128;
constexpr int NCORE_M = 48;
constexpr int NCM = 8;                  // orders per chunk
constexpr size_t kMNodeBytes = 64;      // p w (16), s2, sin xi, and the cos / sin recurrence state (4 x 8)

struct NearMfieSmem {
    // Gb [NTPB][3][NCM] double2, W [NTPB][24] double, Prim [24][M+1] double2
    static size_t bytes(int Mo) {
        return sizeof(double2) * (size_t)NTPB * 3 * NCM + sizeof(double) * (size_t)NTPB * 24 +
               sizeof(double2) * 24 * (size_t)Mo;
    }
};

// accumulate p w {cos(n xi), s2 cos(n xi), sin(xi) sin(n xi)}, n = n0..n0+NCM-1,
// from the recurrence state (cos, sin of (n0-1) xi and n0 xi), which is advanced
__device__ __forceinline__ void project3(double2 (&acc)[3][NCM], double2 p, double s2, double sx,
                                         double &cm1, double &c0, double &sm1, double &s0)
{
    const double c1 = 1.0 - 2.0 * s2;            // cos(xi)
    const double qre = p.x * s2, qim = p.y * s2;
    const double ure = p.x * sx, uim = p.y * sx;
#pragma unroll
    for (int n = 0; n < NCM; ++n) {
        acc[0][n].x = fma(p.x, c0, acc[0][n].x); acc[0][n].y = fma(p.y, c0, acc[0][n].y);
        acc[1][n].x = fma(qre, c0, acc[1][n].x); acc[1][n].y = fma(qim, c0, acc[1][n].y);
        acc[2][n].x = fma(ure, s0, acc[2][n].x); acc[2][n].y = fma(uim, s0, acc[2][n].y);
        const double cn = 2.0 * c1 * c0 - cm1; cm1 = c0; c0 = cn;
        const double sn = 2.0 * c1 * s0 - sm1; sm1 = s0; s0 = sn;
    }
}

template <bool IBC, bool CK = false>
__global__ void __launch_bounds__(NTPB, 2)
near_mfie_kernel(int N, int Nn, int M, double k, double ki, double sc_re, double sc_im,
                 const double2 *__restrict__ wsrc,
                 const double *__restrict__ nodes, const double *__restrict__ elem,
                 const double *__restrict__ emass, int n_pairs,
                 const int *__restrict__ pairs, const int *__restrict__ tails,
                 const double *__restrict__ cells, int ncells_total,
                 const double *__restrict__ core_gl, const double *__restrict__ tail_gl, int ntail_total,
                 int nmax, double2 *__restrict__ band, double2 *__restrict__ Z, long long ldz,
                 long long mode_stride, unsigned char *__restrict__ scratch, int *__restrict__ status)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Mo = M + 1;
    double2 *Gb = reinterpret_cast<double2 *>(smem_raw);
    double *W = reinterpret_cast<double *>(Gb + NTPB * 3 * NCM);
    double2 *Prim = reinterpret_cast<double2 *>(W + NTPB * 24);
    const int tid = threadIdx.x;

    const size_t plane = (size_t)nmax * NTPB;
    double2 *gP = reinterpret_cast<double2 *>(scratch + (size_t)blockIdx.x * plane * kMNodeBytes);
    double *gS2 = reinterpret_cast<double *>(gP + plane);
    double *gSx = gS2 + plane;
    double *gCm = gSx + plane;
    double *gC0 = gCm + plane;
    double *gSm = gC0 + plane;
    double *gS0 = gSm + plane;

    constexpr int NOUT = (24 * NCM + NTPB - 1) / NTPB;
    const int nchunk = (Mo + NCM - 1) / NCM;
    const double ik4pi = 1.0 / (4.0 * GB_PI);

    for (int pi = blockIdx.x; pi < n_pairs; pi += gridDim.x) {
        const int e = pairs[4 * pi + 0], f = pairs[4 * pi + 1];
        const int coff = pairs[4 * pi + 2], ncell = pairs[4 * pi + 3];
        const int toff = tails[2 * pi + 0], ntail = tails[2 * pi + 1];
        const int nn = NCORE_M + ntail;
        if (nn > nmax) {
            if (tid == 0) atomicExch(status, 1);
            continue;
        }
        const double rho_e0 = nodes[2 * e], z_e0 = nodes[2 * e + 1];
        const double drho_e = nodes[2 * e + 2] - rho_e0, dz_e = nodes[2 * e + 3] - z_e0;
        const double rho_f0 = nodes[2 * f], z_f0 = nodes[2 * f + 1];
        const double drho_f = nodes[2 * f + 2] - rho_f0, dz_f = nodes[2 * f + 3] - z_f0;
        const double Le = elem[e], Lf = elem[f];
        const double tre = elem[N + e], tze = elem[2 * N + e];
        const double trf = elem[N + f], tzf = elem[2 * N + f];

        __syncthreads();                     // the previous pair has finished reading Prim
        for (int i = tid; i < 24 * Mo; i += NTPB) Prim[i] = make_double2(0.0, 0.0);

        const int nbatch = (ncell + NTPB - 1) / NTPB;
        for (int bt = 0; bt < nbatch; ++bt) {
            const int c = bt * NTPB + tid;
            const bool valid = c < ncell;
            double wl[24];
#pragma unroll
            for (int i = 0; i < 24; ++i) wl[i] = 0.0;
            if (valid) {
                const double s = cells[coff + c];
                const double sp = cells[ncells_total + coff + c];
                const double wc = cells[2 * ncells_total + coff + c];
                const double rp = rho_e0 + s * drho_e, zp = z_e0 + s * dz_e;
                const double rq = rho_f0 + sp * drho_f, zq = z_f0 + sp * dz_f;
                const double w = wc * Le * Lf;
                const double dr = rp - rq, dz = zp - zq;
                const double d2 = dr * dr + dz * dz;
                const double rr4 = 4.0 * rp * rq;
                // near bracket grid (bor_kernels.py:380-404): s0 = 1 on the axis
                const double d = sqrt(fmax(d2, 1e-300));
                const double a = fmax(sqrt(fmax(rr4, 0.0)), 1e-300);
                const double da = d / a;
                const double s0 = (rr4 <= 1e-30) ? 1.0 : fmin(0.25, 20.0 * da);
                const double vmax = asinh(s0 / da);
                for (int i = 0; i < NCORE_M; ++i) {
                    const double v = core_gl[i] * vmax;
                    const double wv = core_gl[NCORE_M + i] * vmax;
                    const double sh = sinh(v), chv = cosh(v);
                    const double sv = fmin(da * sh, 1.0);
                    const double cv = sqrt(fmax(1.0 - sv * sv, 0.0));       // cos(xi/2)
                    const double dxi = 2.0 * da * chv / sqrt(fmax(1.0 - sv * sv, 1e-15));
                    const double R = fmax(sqrt(d * d + (a * sv) * (a * sv)), 1e-300);
                    const double kr = k * R;
                    double sn, cs;
                    sincos(kr, &sn, &cs);
                    const double ir = 1.0 / R;
                    const double amp = 2.0 * wv * dxi * ik4pi * ir * ir * ir;   // x2: +xi and -xi
                    const size_t q = (size_t)i * NTPB + tid;
                    const double sx = 2.0 * sv * cv;
                    if constexpr (CK) {
                        // (1 + j k R) e^{-j k R} with k = k_r + j k_i:
                        // (1 - k_i R + j k_r R) e^{k_i R} (cos k_r R - j sin k_r R)
                        const double u = 1.0 - ki * R, ea = amp * exp(ki * R);
                        gP[q] = make_double2((u * cs + kr * sn) * ea, (kr * cs - u * sn) * ea);
                    } else {
                        gP[q] = make_double2(fma(kr, sn, cs) * amp, fma(kr, cs, -sn) * amp);
                    }
                    gS2[q] = sv * sv;
                    gSx[q] = sx;
                    gCm[q] = 1.0 - 2.0 * sv * sv; gC0[q] = 1.0;    // cos(-xi), cos(0)
                    gSm[q] = -sx; gS0[q] = 0.0;                    // sin(-xi), sin(0)
                }
                const double xi0 = 2.0 * asin(fmin(s0, 1.0));
                const double span = GB_PI - xi0;
                const bool std_tail = s0 == 0.25;          // tabulated half-angle nodes
                for (int i = 0; i < ntail; ++i) {
                    const double wt = tail_gl[ntail_total + toff + i] * span;
                    double st, ct;
                    if (std_tail) {
                        st = tail_gl[2 * ntail_total + toff + i];
                        ct = tail_gl[3 * ntail_total + toff + i];
                    } else {
                        sincos(0.5 * (xi0 + tail_gl[toff + i] * span), &st, &ct);
                    }
                    const double R = fmax(sqrt(d * d + (a * st) * (a * st)), 1e-300);
                    const double kr = k * R;
                    double sn, cs;
                    sincos(kr, &sn, &cs);
                    const double ir = 1.0 / R;
                    const double amp = 2.0 * wt * ik4pi * ir * ir * ir;
                    const size_t q = (size_t)(NCORE_M + i) * NTPB + tid;
                    const double sx = 2.0 * st * ct;
                    if constexpr (CK) {
                        const double u = 1.0 - ki * R, ea = amp * exp(ki * R);
                        gP[q] = make_double2((u * cs + kr * sn) * ea, (kr * cs - u * sn) * ea);
                    } else {
                        gP[q] = make_double2(fma(kr, sn, cs) * amp, fma(kr, cs, -sn) * amp);
                    }
                    gS2[q] = st * st;
                    gSx[q] = sx;
                    gCm[q] = 1.0 - 2.0 * st * st; gC0[q] = 1.0;
                    gSm[q] = -sx; gS0[q] = 0.0;
                }
                double cf[6];
                bracket_coefs<IBC>(rp, zp, tre, tze, rq, zq, trf, tzf, cf);
                const double Tp[2] = {1.0 - s, s}, Tq[2] = {1.0 - sp, sp};
                const double rr = 2.0 * GB_PI * rp * rq * w;
#pragma unroll
                for (int ab = 0; ab < 4; ++ab) {
                    const double wab = Tp[ab >> 1] * Tq[ab & 1] * rr;
#pragma unroll
                    for (int kk = 0; kk < 6; ++kk) wl[kk * 4 + ab] = wab * cf[kk];
                }
            }
            __syncthreads();                 // the previous batch's GEMM has finished reading W
#pragma unroll
            for (int i = 0; i < 24; ++i) W[tid * 24 + i] = wl[i];
            const int cnt = min(NTPB, ncell - bt * NTPB);

            for (int ch = 0; ch < nchunk; ++ch) {
                const int n0 = ch * NCM;
                double2 acc[3][NCM];
#pragma unroll
                for (int t = 0; t < 3; ++t)
#pragma unroll
                    for (int n = 0; n < NCM; ++n) acc[t][n] = make_double2(0.0, 0.0);
                if (valid) {
                    for (int v = 0; v < nn; ++v) {
                        const size_t q = (size_t)v * NTPB + tid;
                        double cm1 = gCm[q], c0 = gC0[q], sm1 = gSm[q], s0 = gS0[q];
                        project3(acc, gP[q], gS2[q], gSx[q], cm1, c0, sm1, s0);
                        if (ch + 1 < nchunk) { gCm[q] = cm1; gC0[q] = c0; gSm[q] = sm1; gS0[q] = s0; }
                    }
                }
                __syncthreads();             // the previous chunk's GEMM has finished reading Gb
#pragma unroll
                for (int t = 0; t < 3; ++t)
#pragma unroll
                    for (int n = 0; n < NCM; ++n) Gb[(tid * 3 + t) * NCM + n] = acc[t][n];
                __syncthreads();
                // GEMM: Prim(kind, ab, n0 + n) += sum_t W[t][kind, ab] Gb[t][src(kind)][n],
                // src = C[p] for kinds 0, 2; C[p s2] for 1, 3; S for 4, 5
#pragma unroll
                for (int r = 0; r < NOUT; ++r) {
                    const int o = tid + r * NTPB;
                    if (o < 24 * NCM) {
                        const int c24 = o / NCM, n = o % NCM;
                        const int kind = c24 >> 2;
                        const int src = kind >= 4 ? 2 : (kind & 1);
                        double2 sacc = make_double2(0.0, 0.0);
                        for (int t = 0; t < cnt; ++t) {
                            const double wv = W[t * 24 + c24];
                            const double2 gv = Gb[(t * 3 + src) * NCM + n];
                            sacc.x = fma(wv, gv.x, sacc.x);
                            sacc.y = fma(wv, gv.y, sacc.y);
                        }
                        if (n0 + n < Mo) {
                            double2 &pr = Prim[c24 * Mo + n0 + n];
                            pr.x += sacc.x;
                            pr.y += sacc.y;
                        }
                    }
                }
            }
        }
        __syncthreads();

        // blocks: Z_M = M/2 - K (MFIE) or Z_s(f) (M/2 + B) (IBC);
        // K_tt = O0 + O1, K_ff = O2 + O3, K_tf = -j O4, K_ft = -j O5
        double s_re = sc_re, s_im = sc_im;
        if (IBC && wsrc) {
            const double2 w = wsrc[f];
            s_re = sc_re * w.x - sc_im * w.y;
            s_im = sc_re * w.y + sc_im * w.x;
        }
        for (int job = tid; job < Mo * 16; job += NTPB) {
            const int m = job / 16, blk = (job / 4) % 4, ab = job % 4;
            const int a = ab >> 1, b = ab & 1;
            double2 K;
            if (blk == 0 || blk == 3) {
                const int k0 = blk == 0 ? 0 : 2;
                const double2 u = Prim[(k0 * 4 + ab) * Mo + m], v = Prim[((k0 + 1) * 4 + ab) * Mo + m];
                K = make_double2(u.x + v.x, u.y + v.y);
            } else {
                const double2 u = Prim[((blk == 1 ? 4 : 5) * 4 + ab) * Mo + m];
                K = make_double2(u.y, -u.x);
            }
            const double mh = (e == f && (blk == 0 || blk == 3)) ? 0.5 * emass[4 * e + ab] : 0.0;
            double sv2[2];
            bracket_entry<IBC>(K.x, K.y, mh, s_re, s_im, sv2);
            const double2 sv = make_double2(sv2[0], sv2[1]);
            const int i = e + a, j = f + b;
            if (band) {
                double2 *dst = band + (((size_t)m * 4 + blk) * Nn + i) * 5 + (j - i + 2);
                catomic_add(dst, sv);
            } else {
                const long long row = i + (blk >> 1) * Nn, col = j + (blk & 1) * Nn;
                catomic_add(Z + (size_t)m * mode_stride + row * ldz + col, sv);
            }
        }
    }
}

template <class R, bool IBC, bool CK = false>
int launch_far_bracket(int N, int M, int nxi, double k, double sre, double sim, const double *geo,
                       const double *tab, const double *sin2, const double *wsrc, void *Z, long long ldz,
                       long long ms, cudaStream_t st, double ki = 0.0)
{
    const size_t smem = MfieSmem<R>::bytes();
    auto kern = far_mfie_kernel<R, IBC, CK>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("far_mfie: smem attribute");
    const int fgroups = (N + MEPB - 1) / MEPB;
    const int nchunks = (M + 1 + MNOB - 1) / MNOB;
    dim3 grid((unsigned)(N * fgroups), (unsigned)nchunks);
    kern<<<grid, MTPB, smem, st>>>(N, N + 1, M, nxi / 2, k, sre, sim, geo, tab, sin2,
                                   reinterpret_cast<const double2 *>(wsrc),
                                   reinterpret_cast<double2 *>(Z), ldz, ms, ki);
    return check_launch(CK ? "far_ibc (complex k)" : IBC ? "far_ibc" : "far_mfie");
}

template <bool IBC>
int far_bracket(int prec, int n_elem, int m_max, int nxi, double k, double sre, double sim,
                const double *geo, const double *tab, const double *sin2, const double *wsrc,
                void *Z, long long ldz, long long ms, void *stream)
{
    if (n_elem < 3 || m_max < 0 || nxi < 2 || (nxi & 1) || !geo || !tab || !sin2 || !Z ||
        ldz < 2LL * (n_elem + 1) || ms < ldz * 2LL * (n_elem + 1) || !(k > 0.0))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (prec == GHOST_BOR_F32)
        return launch_far_bracket<float, IBC>(n_elem, m_max, nxi, k, sre, sim, geo, tab, sin2, wsrc, Z, ldz, ms, st);
    if (prec == GHOST_BOR_F64)
        return launch_far_bracket<double, IBC>(n_elem, m_max, nxi, k, sre, sim, geo, tab, sin2, wsrc, Z, ldz, ms, st);
    return GHOST_BOR_EINVAL;
}

template <bool IBC, bool CK = false>
int near_bracket(int n_elem, int m_max, double k, double sre, double sim, const double *wsrc,
                 const double *nodes, const double *elem, const double *emass, int n_pairs, const int *pairs,
                 const int *tails, const double *cells, int n_cells_total, const double *core_gl,
                 const double *tail_gl, int n_tail_total, double *band, void *Z, long long ldz, long long ms,
                 int n_tail_max, void *work, long long work_bytes, long long work_need, void *stream,
                 double ki = 0.0)
{
    if (n_elem < 1 || m_max < 0 || n_pairs < 1 || !nodes || !elem || !emass || !pairs || !tails ||
        !cells || !core_gl || !tail_gl || !(k > 0.0) || n_tail_max < 0 || !work ||
        (reinterpret_cast<uintptr_t>(work) & 255) || work_bytes < work_need)
        return GHOST_BOR_EINVAL;
    if (!band && (!Z || ldz < 2LL * (n_elem + 1))) return GHOST_BOR_EINVAL;
    const size_t smem = NearMfieSmem::bytes(m_max + 1);
    if (smem > 227 * 1024) return GHOST_BOR_EUNSUPPORTED;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    auto kern = near_mfie_kernel<IBC, CK>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("near_mfie: smem attribute");
    int *status = reinterpret_cast<int *>(work);
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return check_launch("near_mfie: memset");
    const int grid = n_pairs < near_grid() ? n_pairs : near_grid();
    kern<<<grid, NTPB, smem, st>>>(
        n_elem, n_elem + 1, m_max, k, ki, sre, sim, reinterpret_cast<const double2 *>(wsrc), nodes, elem, emass,
        n_pairs, pairs, tails, cells, n_cells_total, core_gl, tail_gl, n_tail_total, NCORE_M + n_tail_max,
        reinterpret_cast<double2 *>(band), reinterpret_cast<double2 *>(Z), ldz, ms,
        reinterpret_cast<unsigned char *>(work) + 256, status);
    return check_launch(CK ? "near_ibc (complex k)" : IBC ? "near_ibc" : "near_mfie");
}

}  // namespace
}  // namespace gb

extern "C" int ghost_bor_far_mfie(int prec, int n_elem, int m_max, int nxi, double k,
                                  double scale_re, double scale_im,
                                  const double *geo, const double *tab, const double *sin2,
                                  void *Z, long long ldz, long long mode_stride, void *stream)
{
    return gb::far_bracket<false>(prec, n_elem, m_max, nxi, k, scale_re, scale_im, geo, tab, sin2, nullptr,
                                  Z, ldz, mode_stride, stream);
}

extern "C" int ghost_bor_far_ibc(int prec, int n_elem, int m_max, int nxi, double k,
                                 double scale_re, double scale_im, const double *zs_elem,
                                 const double *geo, const double *tab, const double *sin2,
                                 void *Z, long long ldz, long long mode_stride, void *stream)
{
    return gb::far_bracket<true>(prec, n_elem, m_max, nxi, k, scale_re, scale_im, geo, tab, sin2, zs_elem,
                                 Z, ldz, mode_stride, stream);
}

extern "C" long long ghost_bor_near_mfie_workspace(int n_tail_max)
{
    if (n_tail_max < 0) return -1;
    return 256 + (long long)gb::near_grid() * gb::NTPB * (gb::NCORE_M + n_tail_max) * (long long)gb::kMNodeBytes;
}

extern "C" int ghost_bor_near_mfie(int n_elem, int m_max, double k, double scale_re, double scale_im,
                                   const double *nodes, const double *elem, const double *emass,
                                   int n_pairs, const int *pairs, const int *tails,
                                   const double *cells, int n_cells_total,
                                   const double *core_gl, const double *tail_gl, int n_tail_total,
                                   double *band, void *Z, long long ldz, long long mode_stride,
                                   int n_tail_max, void *work, long long work_bytes, void *stream)
{
    return gb::near_bracket<false>(n_elem, m_max, k, scale_re, scale_im, nullptr, nodes, elem, emass, n_pairs,
                                   pairs, tails, cells, n_cells_total, core_gl, tail_gl, n_tail_total, band, Z,
                                   ldz, mode_stride, n_tail_max, work, work_bytes,
                                   ghost_bor_near_mfie_workspace(n_tail_max), stream);
}

extern "C" int ghost_bor_near_ibc(int n_elem, int m_max, double k, double scale_re, double scale_im,
                                  const double *zs_elem, const double *nodes, const double *elem,
                                  const double *emass, int n_pairs, const int *pairs, const int *tails,
                                  const double *cells, int n_cells_total,
                                  const double *core_gl, const double *tail_gl, int n_tail_total,
                                  double *band, void *Z, long long ldz, long long mode_stride,
                                  int n_tail_max, void *work, long long work_bytes, void *stream)
{
    return gb::near_bracket<true>(n_elem, m_max, k, scale_re, scale_im, zs_elem, nodes, elem, emass, n_pairs,
                                  pairs, tails, cells, n_cells_total, core_gl, tail_gl, n_tail_total, band, Z,
                                  ldz, mode_stride, n_tail_max, work, work_bytes,
                                  ghost_bor_near_mfie_workspace(n_tail_max), stream);
}

extern "C" int ghost_bor_far_ibc_ck(int n_elem, int m_max, int nxi, double k_re, double k_im,
                                    double scale_re, double scale_im, const double *zs_elem,
                                    const double *geo, const double *tab, const double *sin2,
                                    void *Z, long long ldz, long long mode_stride, void *stream)
{
    using namespace gb;
    if (n_elem < 3 || m_max < 0 || nxi < 2 || (nxi & 1) || !geo || !tab || !sin2 || !Z ||
        ldz < 2LL * (n_elem + 1) || mode_stride < ldz * 2LL * (n_elem + 1) || !(k_re > 0.0) ||
        !(k_im <= 0.0) || !isfinite(k_re) || !isfinite(k_im))
        return GHOST_BOR_EINVAL;
    return launch_far_bracket<double, true, true>(n_elem, m_max, nxi, k_re, scale_re, scale_im, geo, tab, sin2,
                                                  zs_elem, Z, ldz, mode_stride,
                                                  reinterpret_cast<cudaStream_t>(stream), k_im);
}

extern "C" int ghost_bor_near_ibc_ck(int n_elem, int m_max, double k_re, double k_im,
                                     double scale_re, double scale_im, const double *zs_elem,
                                     const double *nodes, const double *elem, const double *emass,
                                     int n_pairs, const int *pairs, const int *tails,
                                     const double *cells, int n_cells_total,
                                     const double *core_gl, const double *tail_gl, int n_tail_total,
                                     double *band, void *Z, long long ldz, long long mode_stride,
                                     int n_tail_max, void *work, long long work_bytes, void *stream)
{
    if (!(k_im <= 0.0) || !isfinite(k_im)) return GHOST_BOR_EINVAL;
    return gb::near_bracket<true, true>(n_elem, m_max, k_re, scale_re, scale_im, zs_elem, nodes, elem, emass,
                                        n_pairs, pairs, tails, cells, n_cells_total, core_gl, tail_gl,
                                        n_tail_total, band, Z, ldz, mode_stride, n_tail_max, work, work_bytes,
                                        ghost_bor_near_mfie_workspace(n_tail_max), stream, k_im);
}
