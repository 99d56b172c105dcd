// far_fill.cu -- fused EFIE far-field impedance fill for all azimuthal modes.
//
// Replaces the reference's streamed far assembly (bor_streaming.py:220-268
// tile sweep, :320-341 sampling + FFT, :343-349 near zeroing, :352-376
// contraction, :388-407 per-mode combination) and its C sampler
// (bor_stream_kernel.c:26-48).
//
// One CTA = one test element e x EPB source elements f.  Each of the 16
// threads of an element pair owns one Gauss-point pair (g, h) and
//   1. samples g(xi_j) = exp(-j k R)/(4 pi R) on the HALF azimuth grid
//      xi_j = pi j / h, j = 0..h (h = n_xi/2; g is even in xi, so this is the
//      reference's full-grid trapezoid rule folded in two),
//   2. accumulates the even DCT  G_n = sum_j dct[j][n] g_j  for a chunk of
//      NO orders in registers (the FFT of the reference restricted to the
//      orders that are used),
// then the CTA contracts the 4x4 point pairs with the nodal Galerkin weights
// into five order primitives (11, dd, ds, sd, ss; the rr/zz/r1/1r primitives
// of the reference are tangent multiples of 11 because tangents are constant
// per element), combines orders |m-1|, m, m+1 into the four mode-m blocks
// and adds scale * block into Z[m].
//
// FP32 path: R^2, R and k R are carried as double-float (hi + lo) so the
// phase is accurate to ~3e-7 rad before the FP32 sin/cos, independent of kR.
#include "common.cuh"

namespace gb {
namespace {

constexpr int EPB = 8;            // element pairs per CTA
constexpr int TPB = EPB * 16;     // one thread per Gauss-point pair
constexpr int JC = 32;            // azimuth samples staged per smem chunk

constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr float kTwoPiA = 6.28125f;                                     // 8 significant bits
constexpr float kTwoPiB = (float)(kTwoPi - 6.28125);
constexpr float kTwoPiC = (float)(kTwoPi - 6.28125 - (double)(float)(kTwoPi - 6.28125));
constexpr float kInvTwoPi = (float)(1.0 / kTwoPi);
constexpr float kInv4Pi = (float)(1.0 / (4.0 * GB_PI));

// ---------------------------------------------------------------------------
// per-pair samplers
// ---------------------------------------------------------------------------
template <class R> struct GreenSampler;

template <> struct GreenSampler<double> {
    using S2 = double;          // sin^2 table entry type
    double d2, a2, k;
    __device__ void init(double d2_, double a2_, double k_) { d2 = d2_; a2 = a2_; k = k_; }
    static __device__ __forceinline__ double load_s2(const double *t, int j) { return t[j]; }
    __device__ __forceinline__ double2 operator()(double s2) const {
        double R = sqrt(fma(a2, s2, d2));
        R = fmax(R, 1e-30);
        double sn, cs;
        sincos(k * R, &sn, &cs);
        const double amp = 1.0 / (4.0 * GB_PI * R);
        return make_double2(amp * cs, -amp * sn);
    }
};

template <> struct GreenSampler<float> {
    using S2 = float2;          // (hi, lo) split of sin^2
    float d2h, d2l, a2h, a2l, kh, kl;
    __device__ void init(double d2, double a2, double k) {
        d2h = (float)d2; d2l = (float)(d2 - (double)d2h);
        a2h = (float)a2; a2l = (float)(a2 - (double)a2h);
        kh = (float)k;   kl = (float)(k - (double)kh);
    }
    static __device__ __forceinline__ float2 load_s2(const double *t, int j) {
        const double v = t[j];
        const float hi = (float)v;
        return make_float2(hi, (float)(v - (double)hi));
    }
    __device__ __forceinline__ float2 operator()(float2 s2) const {
        // R^2 = d^2 + a^2 s2 in double-float
        const float p = a2h * s2.x;
        const float pe = fmaf(a2h, s2.x, -p);
        const float t = d2h + p;
        const float bb = t - d2h;
        const float te = (d2h - (t - bb)) + (p - bb);
        const float lo = te + pe + fmaf(a2h, s2.y, a2l * s2.x) + d2l;
        const float R2 = t + lo;
        const float R2l = lo - (R2 - t);
        // R = r + rl from one rsqrt and one Newton-style correction
        const float rs = rsqrtf(R2);
        const float r = R2 * rs;
        const float e = fmaf(-r, r, R2) + R2l;
        const float rl = 0.5f * e * rs;
        // phase k R in double-float, reduced mod 2 pi (Cody-Waite, 3 parts)
        const float ph = kh * r;
        const float phe = fmaf(kh, r, -ph);
        const float phl = phe + fmaf(kh, rl, kl * r);
        const float q = rintf(ph * kInvTwoPi);
        float th = fmaf(-q, kTwoPiA, ph);
        th = fmaf(-q, kTwoPiB, th);
        th = fmaf(-q, kTwoPiC, th);
        th += phl;
        float sn, cs;
        __sincosf(th, &sn, &cs);
        const float amp = rs * kInv4Pi;
        return make_float2(amp * cs, -amp * sn);
    }
};

template <class R> struct SmemLayout {
    // Gs   [EPB][NO][16]  C<R>  per-pair orders, later the mode-local blocks
    // P11s [EPB][NO][4]   C<R>
    // dcts [JC][NO]       R
    // s2s  [JC]           S2
    // wts  [EPB+1][6][4]  R     (index EPB = test element)
    static size_t bytes(int NO) {
        return sizeof(C<R>) * (size_t)EPB * NO * 16 + sizeof(C<R>) * (size_t)EPB * NO * 4 +
               sizeof(R) * (size_t)JC * NO + sizeof(typename GreenSampler<R>::S2) * JC +
               sizeof(R) * (size_t)(EPB + 1) * 24;
    }
};

template <class R, int NO>
__global__ void __launch_bounds__(TPB)
far_efie_kernel(int N, int Nn, int M, int h, double k, double sc_re, double sc_im,
                const double *__restrict__ geo, const double *__restrict__ dct,
                const double *__restrict__ sin2, C<R> *__restrict__ Z,
                long long ldz, long long mode_stride)
{
    using CT = C<R>;
    using Samp = GreenSampler<R>;
    using S2 = typename Samp::S2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT *Gs = reinterpret_cast<CT *>(smem_raw);
    CT *P11s = Gs + EPB * NO * 16;
    R *dcts = reinterpret_cast<R *>(P11s + EPB * NO * 4);
    S2 *s2s = reinterpret_cast<S2 *>(dcts + JC * NO);
    R *wts = reinterpret_cast<R *>(s2s + JC);

    const int P = 4 * N;
    const int fgroups = (N + EPB - 1) / EPB;
    const int e = blockIdx.x / fgroups;
    const int f0 = (blockIdx.x % fgroups) * EPB;
    const int chunk = blockIdx.y;
    const int m0 = chunk * (NO - 2);
    if (m0 > M) return;
    const int m1 = min(M, m0 + NO - 3);
    const int o0 = max(0, m0 - 1);
    const int nord = m1 + 1 - o0 + 1;         // orders o0..m1+1
    const int Mp = M + 2;                     // orders stored in dct rows

    const int tid = threadIdx.x;
    const int ep = tid >> 4;
    const int gh = tid & 15;
    const int f = f0 + ep;
    const bool active = (f < N) && (abs(e - f) >= 2);

    // Galerkin weights: rows 3..8 of geo (T0 w rho, T1 w rho, T0 w, T1 w, dRT0 w, dRT1 w)
    for (int i = tid; i < (EPB + 1) * 24; i += TPB) {
        const int slot = i / 24, r = i % 24;
        const int el = (slot == EPB) ? e : min(f0 + slot, N - 1);
        wts[i] = (R)geo[(size_t)(3 + r / 4) * P + 4 * el + (r % 4)];
    }

    Samp smp;
    {
        const int p = 4 * e + (gh >> 2);
        const int q = 4 * min(f, N - 1) + (gh & 3);
        const double rp = geo[p], zp = geo[P + p];
        const double rq = geo[q], zq = geo[P + q];
        const double dr = rp - rq, dz = zp - zq;
        smp.init(dr * dr + dz * dz, 4.0 * rp * rq, k);
    }

    CT acc[NO];
#pragma unroll
    for (int n = 0; n < NO; ++n) acc[n] = mk<R>(R(0), R(0));

    for (int j0 = 0; j0 <= h; j0 += JC) {
        __syncthreads();
        for (int i = tid; i < JC * NO; i += TPB) {
            const int jj = i / NO, n = i % NO;
            const int j = j0 + jj, o = o0 + n;
            dcts[i] = (j <= h && o < Mp) ? (R)dct[(size_t)j * Mp + o] : R(0);
        }
        for (int jj = tid; jj < JC; jj += TPB) {
            const int j = min(j0 + jj, h);
            s2s[jj] = Samp::load_s2(sin2, j);
        }
        __syncthreads();
        if (active) {
            const int jn = min(JC, h + 1 - j0);
            for (int jj = 0; jj < jn; ++jj) {
                const CT gv = smp(s2s[jj]);
                if constexpr (sizeof(R) == 4) {
                    const float4 *row = reinterpret_cast<const float4 *>(dcts + jj * NO);
#pragma unroll
                    for (int n4 = 0; n4 < NO / 4; ++n4) {
                        const float4 c = row[n4];
                        acc[4 * n4 + 0].x = fmaf(gv.x, c.x, acc[4 * n4 + 0].x);
                        acc[4 * n4 + 0].y = fmaf(gv.y, c.x, acc[4 * n4 + 0].y);
                        acc[4 * n4 + 1].x = fmaf(gv.x, c.y, acc[4 * n4 + 1].x);
                        acc[4 * n4 + 1].y = fmaf(gv.y, c.y, acc[4 * n4 + 1].y);
                        acc[4 * n4 + 2].x = fmaf(gv.x, c.z, acc[4 * n4 + 2].x);
                        acc[4 * n4 + 2].y = fmaf(gv.y, c.z, acc[4 * n4 + 2].y);
                        acc[4 * n4 + 3].x = fmaf(gv.x, c.w, acc[4 * n4 + 3].x);
                        acc[4 * n4 + 3].y = fmaf(gv.y, c.w, acc[4 * n4 + 3].y);
                    }
                } else {
                    const double2 *row = reinterpret_cast<const double2 *>(dcts + jj * NO);
#pragma unroll
                    for (int n2 = 0; n2 < NO / 2; ++n2) {
                        const double2 c = row[n2];
                        acc[2 * n2 + 0].x = fma(gv.x, c.x, acc[2 * n2 + 0].x);
                        acc[2 * n2 + 0].y = fma(gv.y, c.x, acc[2 * n2 + 0].y);
                        acc[2 * n2 + 1].x = fma(gv.x, c.y, acc[2 * n2 + 1].x);
                        acc[2 * n2 + 1].y = fma(gv.y, c.y, acc[2 * n2 + 1].y);
                    }
                }
            }
        }
    }

    // spill per-pair orders to smem: Gs[ep][n][gh]
#pragma unroll
    for (int n = 0; n < NO; ++n) Gs[(ep * NO + n) * 16 + gh] = acc[n];
    __syncthreads();

    const R ik2 = R(1.0 / (k * k));
    // contraction jobs (ep, n): five primitives per order
    for (int job = tid; job < EPB * nord; job += TPB) {
        const int jep = job / nord, n = job % nord;
        const int ff = f0 + jep;
        if (ff >= N || abs(e - ff) < 2) continue;
        CT G[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) G[i] = Gs[(jep * NO + n) * 16 + i];
        const R *wt = wts + EPB * 24;      // test element weights
        const R *ws = wts + jep * 24;      // source element weights
        // right contraction: GR_x[g][b] = sum_h G[g][h] Rx[b][h]
        CT GR1[8], GRs[8], GRd[8];
#pragma unroll
        for (int g = 0; g < 4; ++g)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                CT a1 = mk<R>(0, 0), as = mk<R>(0, 0), ad = mk<R>(0, 0);
#pragma unroll
                for (int hq = 0; hq < 4; ++hq) {
                    const CT gv = G[g * 4 + hq];
                    const R w1 = ws[(0 + b) * 4 + hq], wsv = ws[(2 + b) * 4 + hq], wd = ws[(4 + b) * 4 + hq];
                    a1.x = fma(gv.x, w1, a1.x); a1.y = fma(gv.y, w1, a1.y);
                    as.x = fma(gv.x, wsv, as.x); as.y = fma(gv.y, wsv, as.y);
                    ad.x = fma(gv.x, wd, ad.x); ad.y = fma(gv.y, wd, ad.y);
                }
                GR1[g * 2 + b] = a1; GRs[g * 2 + b] = as; GRd[g * 2 + b] = ad;
            }
        const int o = o0 + n;
        const R tze = (R)geo[(size_t)10 * P + 4 * e], tzf = (R)geo[(size_t)10 * P + 4 * ff];
        const R fm = R(o) * ik2;          // jm/k^2 magnitude
        const R fm2 = R(o) * R(o) * ik2;  // m^2/k^2
        CT *zl = Gs + (jep * NO + n) * 16;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                CT p11 = mk<R>(0, 0), pdd = mk<R>(0, 0), pds = mk<R>(0, 0), psd = mk<R>(0, 0), pss = mk<R>(0, 0);
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    const R l1 = wt[(0 + a) * 4 + g], ls = wt[(2 + a) * 4 + g], ld = wt[(4 + a) * 4 + g];
                    const CT r1 = GR1[g * 2 + b], rsv = GRs[g * 2 + b], rd = GRd[g * 2 + b];
                    p11.x = fma(l1, r1.x, p11.x); p11.y = fma(l1, r1.y, p11.y);
                    pdd.x = fma(ld, rd.x, pdd.x); pdd.y = fma(ld, rd.y, pdd.y);
                    pds.x = fma(ld, rsv.x, pds.x); pds.y = fma(ld, rsv.y, pds.y);
                    psd.x = fma(ls, rd.x, psd.x); psd.y = fma(ls, rd.y, psd.y);
                    pss.x = fma(ls, rsv.x, pss.x); pss.y = fma(ls, rsv.y, pss.y);
                }
                const int ab = a * 2 + b;
                P11s[(jep * NO + n) * 4 + ab] = p11;
                // mode-local parts (mode m = o)
                const R tt = tze * tzf;
                zl[0 * 4 + ab] = mk<R>(tt * p11.x - ik2 * pdd.x, tt * p11.y - ik2 * pdd.y);
                zl[1 * 4 + ab] = mk<R>(fm * pds.y, -fm * pds.x);       // -(j o/k^2) pds
                zl[2 * 4 + ab] = mk<R>(-fm * psd.y, fm * psd.x);       // +(j o/k^2) psd
                zl[3 * 4 + ab] = mk<R>(-fm2 * pss.x, -fm2 * pss.y);
            }
    }
    __syncthreads();

    // mode combination + accumulation into Z[m]
    const int nmodes = m1 - m0 + 1;
    const R sre = (R)sc_re, sim = (R)sc_im;
    for (int job = tid; job < EPB * nmodes; job += TPB) {
        const int jep = job / nmodes, m = m0 + job % nmodes;
        const int ff = f0 + jep;
        if (ff >= N || abs(e - ff) < 2) continue;
        const int nl = abs(m - 1) - o0, nm = m - o0, nh = m + 1 - o0;
        const CT *zl = Gs + (jep * NO + nm) * 16;
        const R tre = (R)geo[(size_t)9 * P + 4 * e], trf = (R)geo[(size_t)9 * P + 4 * ff];
        CT *Zm = Z + (size_t)m * mode_stride;
#pragma unroll
        for (int ab = 0; ab < 4; ++ab) {
            const int a = ab >> 1, b = ab & 1;
            const CT lo = P11s[(jep * NO + nl) * 4 + ab];
            const CT hi = P11s[(jep * NO + nh) * 4 + ab];
            const CT S = cadd(lo, hi), D = csub(lo, hi);
            CT blk[4];
            const R half = R(0.5);
            blk[0] = cadd(mk<R>(half * tre * trf * S.x, half * tre * trf * S.y), zl[0 * 4 + ab]);
            blk[1] = cadd(mk<R>(half * tre * D.y, -half * tre * D.x), zl[1 * 4 + ab]);   // t_rho(e) D/(2j)
            blk[2] = cadd(mk<R>(-half * trf * D.y, half * trf * D.x), zl[2 * 4 + ab]);   // -t_rho(f) D/(2j)
            blk[3] = cadd(mk<R>(half * S.x, half * S.y), zl[3 * 4 + ab]);
            const long long r0 = e + a, c0 = ff + b;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const long long row = r0 + (q >> 1) * Nn, col = c0 + (q & 1) * Nn;
                const CT v = mk<R>(sre * blk[q].x - sim * blk[q].y, sre * blk[q].y + sim * blk[q].x);
                catomic_add(Zm + row * ldz + col, v);
            }
        }
    }
}

template <class R, int NO>
int launch_far(int N, int M, int nxi, double k, double sre, double sim, const double *geo,
               const double *dct, const double *sin2, void *Z, long long ldz, long long ms,
               cudaStream_t st)
{
    const size_t smem = SmemLayout<R>::bytes(NO);
    auto kern = far_efie_kernel<R, NO>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("far_efie: smem attribute");
    const int fgroups = (N + EPB - 1) / EPB;
    const int nchunks = (M + 1 + (NO - 2) - 1) / (NO - 2);
    dim3 grid((unsigned)(N * fgroups), (unsigned)nchunks);
    kern<<<grid, TPB, smem, st>>>(N, N + 1, M, nxi / 2, k, sre, sim, geo, dct, sin2,
                                  reinterpret_cast<C<R> *>(Z), ldz, ms);
    return check_launch("far_efie");
}

}  // namespace
}  // namespace gb

extern "C" int ghost_bor_far_efie(int prec, int n_elem, int m_max, int nxi, double k,
                                  double scale_re, double scale_im,
                                  const double *geo, const double *dct, const double *sin2,
                                  void *Z, long long ldz, long long mode_stride, void *stream)
{
    using namespace gb;
    if (n_elem < 3 || m_max < 0 || nxi < 2 || (nxi & 1) || !geo || !dct || !sin2 || !Z ||
        ldz < 2LL * (n_elem + 1) || mode_stride < ldz * 2LL * (n_elem + 1) || !(k > 0.0))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (prec == GHOST_BOR_F32) {
        if (m_max + 1 <= 30) return launch_far<float, 32>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, st);
        return launch_far<float, 64>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, st);
    }
    if (prec == GHOST_BOR_F64) {
        if (m_max + 1 <= 14) return launch_far<double, 16>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, st);
        return launch_far<double, 32>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, st);
    }
    return GHOST_BOR_EINVAL;
}
