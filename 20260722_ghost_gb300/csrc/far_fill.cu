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
// Precision: the sampling and the DCT (all but a few percent of the flops)
// run in the requested precision; contraction, mode combination and the
// node accumulation always run in FP64 and Z is complex double.  The EFIE
// scalar-potential entries of a node pair are double differences of the
// element-pair contributions (the two elements at a node carry charges of
// opposite sign), which cancels ~(1/kL)^2 ~ 30x at 30 elements per wavelength,
// so any rounding before the node sum is amplified by that factor.  In the
// FP32 path R^2, R and k R are carried as double-float so the phase is exact
// to ~1e-7 rad before an accurate sincosf, and the DCT is summed in blocks
// of 8 samples folded in with Kahan compensation.
#include "common.cuh"

namespace gb {
namespace {

constexpr int EPB = 8;            // element pairs per CTA
constexpr int TPB = EPB * 16;     // one thread per Gauss-point pair
constexpr int JC = 32;            // azimuth samples staged per smem chunk

constexpr double kTwoPi = 6.283185307179586476925286766559;
// 2 pi = A + B + C; A (8 bits) and B (12 bits) are short enough that q*A and
// q*B are exact in FP32 for every reduction count q < 2^11 (k R < 12800).
constexpr float kTwoPiA = 6.28125f;
constexpr float kTwoPiB = 4059.0f / 2097152.0f;
constexpr float kTwoPiC = (float)(kTwoPi - 6.28125 - 4059.0 / 2097152.0);
constexpr float kInvTwoPi = (float)(1.0 / kTwoPi);

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
        const double amp = 1.0 / R;                  // 1/(4 pi) is folded into the DCT table
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
        // phase k R in double-float (ph + phl), reduced mod 2 pi: ph - q A is
        // exact, the subtraction of q B is made exact with a two-sum, and the
        // remaining small terms form a first-order correction dt.
        const float ph = kh * r;
        const float phe = fmaf(kh, r, -ph);
        const float phl = phe + fmaf(kh, rl, kl * r);
        const float q = rintf(ph * kInvTwoPi);
        const float t1 = fmaf(-q, kTwoPiA, ph);
        const float qb = -q * kTwoPiB;
        const float t2 = t1 + qb;
        const float tb = t2 - t1;
        const float t2e = (t1 - (t2 - tb)) + (qb - tb);
        const float dt = fmaf(-q, kTwoPiC, phl) + t2e;
        float sn, cs;
        sincosf(t2, &sn, &cs);
        const float s1 = fmaf(dt, cs, sn);            // sin(t2 + dt)
        const float c1 = fmaf(-dt, sn, cs);           // cos(t2 + dt)
        // 1/R = 1/(r + rl) from an IEEE reciprocal and a first-order correction
        const float ir = __frcp_rn(r);
        const float amp = ir * fmaf(-rl, ir, 1.0f);  // 1/(4 pi) is folded into the DCT table
        return make_float2(amp * c1, -amp * s1);
    }
};

template <class R> struct SmemLayout {
    // Gs   [EPB][NO][16]  double2  per-pair orders, later the mode-local blocks
    // P11s [EPB][NO][4]   double2
    // dcts [JC][NO]       R
    // s2s  [JC]           S2
    // wts  [EPB+1][6][4]  double   (index EPB = test element)
    static size_t bytes(int NO) {
        return sizeof(double2) * (size_t)EPB * NO * 16 + sizeof(double2) * (size_t)EPB * NO * 4 +
               sizeof(R) * (size_t)JC * NO + sizeof(typename GreenSampler<R>::S2) * JC +
               sizeof(double) * (size_t)(EPB + 1) * 24;
    }
};

template <class R, int NO>
__global__ void __launch_bounds__(TPB)
far_efie_kernel(int N, int Nn, int M, int h, double k, double sc_re, double sc_im,
                const double *__restrict__ geo, const double *__restrict__ dct,
                const double *__restrict__ sin2, double2 *__restrict__ Z,
                long long ldz, long long mode_stride)
{
    using CT = C<R>;
    using Samp = GreenSampler<R>;
    using S2 = typename Samp::S2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *Gs = reinterpret_cast<double2 *>(smem_raw);
    double2 *P11s = Gs + EPB * NO * 16;
    R *dcts = reinterpret_cast<R *>(P11s + EPB * NO * 4);
    S2 *s2s = reinterpret_cast<S2 *>(dcts + JC * NO);
    double *wts = reinterpret_cast<double *>(s2s + JC);

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
        wts[i] = geo[(size_t)(3 + r / 4) * P + 4 * el + (r % 4)];
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

    CT acc[NO];          // running sums
    CT cmp[NO];          // Kahan compensation (FP32 path only)
#pragma unroll
    for (int n = 0; n < NO; ++n) { acc[n] = mk<R>(R(0), R(0)); cmp[n] = mk<R>(R(0), R(0)); }

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
            if constexpr (sizeof(R) == 4) {
                // FP32: sums over blocks of 8 samples, each folded into the
                // running sum with Kahan compensation.  The node-level EFIE
                // entries are double differences of these orders, so their
                // rounding error must stay well below one FP32 ulp.
                for (int jb = 0; jb < jn; jb += 8) {
                    CT cacc[NO];
#pragma unroll
                    for (int n = 0; n < NO; ++n) cacc[n] = mk<R>(R(0), R(0));
                    const int je = min(jb + 8, jn);
                    for (int jj = jb; jj < je; ++jj) {
                        const CT gv = smp(s2s[jj]);
                        const float4 *row = reinterpret_cast<const float4 *>(dcts + jj * NO);
#pragma unroll
                        for (int n4 = 0; n4 < NO / 4; ++n4) {
                            const float4 c = row[n4];
                            cacc[4 * n4 + 0].x = fmaf(gv.x, c.x, cacc[4 * n4 + 0].x);
                            cacc[4 * n4 + 0].y = fmaf(gv.y, c.x, cacc[4 * n4 + 0].y);
                            cacc[4 * n4 + 1].x = fmaf(gv.x, c.y, cacc[4 * n4 + 1].x);
                            cacc[4 * n4 + 1].y = fmaf(gv.y, c.y, cacc[4 * n4 + 1].y);
                            cacc[4 * n4 + 2].x = fmaf(gv.x, c.z, cacc[4 * n4 + 2].x);
                            cacc[4 * n4 + 2].y = fmaf(gv.y, c.z, cacc[4 * n4 + 2].y);
                            cacc[4 * n4 + 3].x = fmaf(gv.x, c.w, cacc[4 * n4 + 3].x);
                            cacc[4 * n4 + 3].y = fmaf(gv.y, c.w, cacc[4 * n4 + 3].y);
                        }
                    }
#pragma unroll
                    for (int n = 0; n < NO; ++n) {
                        const float yx = cacc[n].x - cmp[n].x, yy = cacc[n].y - cmp[n].y;
                        const float tx = acc[n].x + yx, ty = acc[n].y + yy;
                        cmp[n].x = (tx - acc[n].x) - yx;
                        cmp[n].y = (ty - acc[n].y) - yy;
                        acc[n].x = tx;
                        acc[n].y = ty;
                    }
                }
            } else {
                for (int jj = 0; jj < jn; ++jj) {
                    const CT gv = smp(s2s[jj]);
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

    // per-pair orders to smem in FP64: Gs[ep][n][gh] = acc - cmp
#pragma unroll
    for (int n = 0; n < NO; ++n)
        Gs[(ep * NO + n) * 16 + gh] = make_double2((double)acc[n].x - (double)cmp[n].x,
                                                   (double)acc[n].y - (double)cmp[n].y);
    __syncthreads();

    const double ik2 = 1.0 / (k * k);
    // contraction jobs (ep, n): five primitives per order
    for (int job = tid; job < EPB * nord; job += TPB) {
        const int jep = job / nord, n = job % nord;
        const int ff = f0 + jep;
        if (ff >= N || abs(e - ff) < 2) continue;
        double2 G[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) G[i] = Gs[(jep * NO + n) * 16 + i];
        const double *wt = wts + EPB * 24;      // test element weights
        const double *ws = wts + jep * 24;      // source element weights
        // right contraction: GR_x[g][b] = sum_h G[g][h] Rx[b][h]
        double2 GR1[8], GRs[8], GRd[8];
#pragma unroll
        for (int g = 0; g < 4; ++g)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                double2 a1 = make_double2(0, 0), as = make_double2(0, 0), ad = make_double2(0, 0);
#pragma unroll
                for (int hq = 0; hq < 4; ++hq) {
                    const double2 gv = G[g * 4 + hq];
                    const double w1 = ws[(0 + b) * 4 + hq], wsv = ws[(2 + b) * 4 + hq], wd = ws[(4 + b) * 4 + hq];
                    a1.x = fma(gv.x, w1, a1.x); a1.y = fma(gv.y, w1, a1.y);
                    as.x = fma(gv.x, wsv, as.x); as.y = fma(gv.y, wsv, as.y);
                    ad.x = fma(gv.x, wd, ad.x); ad.y = fma(gv.y, wd, ad.y);
                }
                GR1[g * 2 + b] = a1; GRs[g * 2 + b] = as; GRd[g * 2 + b] = ad;
            }
        const int o = o0 + n;
        const double tze = geo[(size_t)10 * P + 4 * e], tzf = geo[(size_t)10 * P + 4 * ff];
        const double fm = o * ik2;          // jm/k^2 magnitude
        const double fm2 = (double)o * o * ik2;  // m^2/k^2
        double2 *zl = Gs + (jep * NO + n) * 16;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b) {
                double2 p11 = make_double2(0, 0), pdd = make_double2(0, 0), pds = make_double2(0, 0), psd = make_double2(0, 0), pss = make_double2(0, 0);
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    const double l1 = wt[(0 + a) * 4 + g], ls = wt[(2 + a) * 4 + g], ld = wt[(4 + a) * 4 + g];
                    const double2 r1 = GR1[g * 2 + b], rsv = GRs[g * 2 + b], rd = GRd[g * 2 + b];
                    p11.x = fma(l1, r1.x, p11.x); p11.y = fma(l1, r1.y, p11.y);
                    pdd.x = fma(ld, rd.x, pdd.x); pdd.y = fma(ld, rd.y, pdd.y);
                    pds.x = fma(ld, rsv.x, pds.x); pds.y = fma(ld, rsv.y, pds.y);
                    psd.x = fma(ls, rd.x, psd.x); psd.y = fma(ls, rd.y, psd.y);
                    pss.x = fma(ls, rsv.x, pss.x); pss.y = fma(ls, rsv.y, pss.y);
                }
                const int ab = a * 2 + b;
                P11s[(jep * NO + n) * 4 + ab] = p11;
                // mode-local parts (mode m = o)
                const double tt = tze * tzf;
                zl[0 * 4 + ab] = make_double2(tt * p11.x - ik2 * pdd.x, tt * p11.y - ik2 * pdd.y);
                zl[1 * 4 + ab] = make_double2(fm * pds.y, -fm * pds.x);       // -(j o/k^2) pds
                zl[2 * 4 + ab] = make_double2(-fm * psd.y, fm * psd.x);       // +(j o/k^2) psd
                zl[3 * 4 + ab] = make_double2(-fm2 * pss.x, -fm2 * pss.y);
            }
    }
    __syncthreads();

    // mode combination + accumulation into Z[m]
    const int nmodes = m1 - m0 + 1;
    const double sre = sc_re, sim = sc_im;
    for (int job = tid; job < EPB * nmodes; job += TPB) {
        const int jep = job / nmodes, m = m0 + job % nmodes;
        const int ff = f0 + jep;
        if (ff >= N || abs(e - ff) < 2) continue;
        const int nl = abs(m - 1) - o0, nm = m - o0, nh = m + 1 - o0;
        const double2 *zl = Gs + (jep * NO + nm) * 16;
        const double tre = geo[(size_t)9 * P + 4 * e], trf = geo[(size_t)9 * P + 4 * ff];
        double2 *Zm = Z + (size_t)m * mode_stride;
#pragma unroll
        for (int ab = 0; ab < 4; ++ab) {
            const int a = ab >> 1, b = ab & 1;
            const double2 lo = P11s[(jep * NO + nl) * 4 + ab];
            const double2 hi = P11s[(jep * NO + nh) * 4 + ab];
            const double2 S = cadd(lo, hi), D = csub(lo, hi);
            double2 blk[4];
            const double half = 0.5;
            blk[0] = cadd(make_double2(half * tre * trf * S.x, half * tre * trf * S.y), zl[0 * 4 + ab]);
            blk[1] = cadd(make_double2(half * tre * D.y, -half * tre * D.x), zl[1 * 4 + ab]);   // t_rho(e) D/(2j)
            blk[2] = cadd(make_double2(-half * trf * D.y, half * trf * D.x), zl[2 * 4 + ab]);   // -t_rho(f) D/(2j)
            blk[3] = cadd(make_double2(half * S.x, half * S.y), zl[3 * 4 + ab]);
            const long long r0 = e + a, c0 = ff + b;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const long long row = r0 + (q >> 1) * Nn, col = c0 + (q & 1) * Nn;
                const double2 v = make_double2(sre * blk[q].x - sim * blk[q].y, sre * blk[q].y + sim * blk[q].x);
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
                                  reinterpret_cast<double2 *>(Z), ldz, ms);
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
        if (m_max + 1 <= 14) return launch_far<float, 16>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, st);
        return launch_far<float, 32>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, st);
    }
    if (prec == GHOST_BOR_F64) {
        if (m_max + 1 <= 14) return launch_far<double, 16>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, st);
        return launch_far<double, 32>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, st);
    }
    return GHOST_BOR_EINVAL;
}
