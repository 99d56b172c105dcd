// far_fill.cu -- fused EFIE far-field impedance fill for all azimuthal modes.
//
// Replaces the reference's streamed far assembly (bor_streaming.py:220-268
// tile sweep, :320-341 sampling + FFT, :343-349 near zeroing, :352-376
// contraction, :388-407 per-mode combination) and its C sampler
// (bor_stream_kernel.c:26-48).
//
// One CTA = one test element e x EPB source elements f = 16 EPB Gauss-point
// pairs (g, h), each served by OG threads that
//   1. sample g(xi_j) = exp(-j k R)/(4 pi R) on the HALF azimuth grid
//      xi_j = pi j / h, j = 0..h (h = n_xi/2; g is even in xi, so this is the
//      reference's full-grid trapezoid rule folded in two), each thread a
//      stride-OG subset of a 32-sample chunk, into shared memory,
//   2. accumulate the even DCT  G_n = sum_j dct[j][n] g_j, each thread for
//      its NT orders, in registers (the FFT of the reference restricted to
//      the orders that are used),
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
#include <type_traits>

#include "common.cuh"
#include "samplers.cuh"
#include "df_math.cuh"

namespace gb {
namespace {

constexpr int TPB = 256;          // threads: Gauss-point pairs (16 EPB) x order groups (OG)
constexpr int JC = 32;            // azimuth samples staged per smem chunk

constexpr int SLAB = 17;              // 16-byte entries per (pair, order) slab of Gs: 16 used + 1 pad
                                      // so that slabs read by neighbouring threads hit distinct banks
// OG order groups (threads sharing one Gauss-point pair) of NT orders each;
// EPB = 16 / OG element pairs per CTA.  OG = 4 for up to 62 orders per launch
// row, OG = 8 (two element pairs per CTA) for up to 126, so that every
// sample is evaluated once for |m| <= 124.

template <class R, int NT, int OG> struct SmemLayout {
    static constexpr int EPB = 16 / OG, PPB = EPB * 16;
    // gsm  [JC][PPB]        C<R>     samples of the current chunk
    // dcts [JC][OG*NT]      R
    // s2s  [JC]             S2
    // Gs   [EPB][OG*NT][SLAB] 16 B   per-pair orders, later the mode-local blocks
    // P11s [EPB][OG*NT][4]  16 B
    // wts  [EPB+1][24]      double ; wtf [EPB+1][24] float2
    static constexpr int NOB = OG * NT;
    static size_t bytes() {
        return sizeof(C<R>) * (size_t)JC * PPB + sizeof(R) * (size_t)JC * NOB +
               sizeof(typename GreenSampler<R>::S2) * JC + 16 * (size_t)EPB * NOB * SLAB +
               16 * (size_t)EPB * NOB * 4 + (sizeof(double) + sizeof(float2)) * (size_t)(EPB + 1) * 24;
    }
};

// CK: complex wave number k + j ki (FP64 only; a lossy medium's interior)
template <class R, int NT, int OG, bool CK = false>
__global__ void __launch_bounds__(TPB, 2)
far_efie_kernel(int N, int Nn, int M, int h, double k, double sc_re, double sc_im,
                const double *__restrict__ geo, const double *__restrict__ dct,
                const double *__restrict__ sin2, double2 *__restrict__ Z,
                long long ldz, long long mode_stride, const unsigned char *__restrict__ emask,
                const float *__restrict__ dct32, double ki)
{
    static_assert(!CK || sizeof(R) == 8, "complex wave numbers on the FP64 path only");
    using CT = C<R>;
    using Samp = typename std::conditional<CK, GreenSamplerC, GreenSampler<R>>::type;
    using S2 = typename Samp::S2;
    constexpr int NOB = OG * NT;
    constexpr int EPB = 16 / OG, PPB = EPB * 16;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT *gsm = reinterpret_cast<CT *>(smem_raw);
    R *dcts = reinterpret_cast<R *>(gsm + JC * PPB);
    S2 *s2s = reinterpret_cast<S2 *>(dcts + JC * NOB);
    double2 *Gs = reinterpret_cast<double2 *>(s2s + JC);
    double2 *P11s = Gs + EPB * NOB * SLAB;
    double *wts = reinterpret_cast<double *>(P11s + EPB * NOB * 4);
    float2 *wtf = reinterpret_cast<float2 *>(wts + (EPB + 1) * 24);

    const int P = 4 * N;
    const int fgroups = (N + EPB - 1) / EPB;
    const int e = blockIdx.x / fgroups;
    const int f0 = (blockIdx.x % fgroups) * EPB;
    const int m0 = blockIdx.y * (NOB - 2);
    if (m0 > M) return;
    // element mask: only pairs with a flagged test or source element (used for
    // the shape-derivative fills of the adjoint gradient)
    if (emask && !emask[e]) {
        bool any = false;
        for (int j = 0; j < EPB; ++j) any |= (f0 + j < N) && emask[f0 + j];
        if (!any) return;
    }
    const int m1 = min(M, m0 + NOB - 3);
    const int o0 = max(0, m0 - 1);
    const int nord = m1 + 1 - o0 + 1;         // orders o0..m1+1
    const int Mp = M + 2;

    const int tid = threadIdx.x;
    const int og = tid / PPB;                 // order group of this thread
    const int pp = tid % PPB;                 // Gauss-point pair of this thread
    const int ep = pp >> 4, gh = pp & 15;
    const int f = f0 + ep;
    const bool active = (f < N) && (abs(e - f) >= 2) && (!emask || emask[e] || emask[f]);

    for (int i = tid; i < (EPB + 1) * 24; i += TPB) {
        const int slot = i / 24, r = i % 24;
        const int el = (slot == EPB) ? e : min(f0 + slot, N - 1);
        const double w = geo[(size_t)(3 + r / 4) * P + 4 * el + (r % 4)];
        wts[i] = w;
        wtf[i] = df_from(w);
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

    CT acc[NT];          // running sums of this thread's NT orders
    CT cmp[NT];          // Kahan compensation (FP32 path only)
#pragma unroll
    for (int n = 0; n < NT; ++n) { acc[n] = mk<R>(R(0), R(0)); cmp[n] = mk<R>(R(0), R(0)); }

    for (int j0 = 0; j0 <= h; j0 += JC) {
        __syncthreads();                      // previous chunk consumed
        for (int i = tid; i < JC * NOB; i += TPB) {
            const int jj = i / NOB, n = i % NOB;
            const int j = j0 + jj, o = o0 + n;
            R t = R(0);
            if (j <= h && o < Mp) {
                if constexpr (sizeof(R) == 4) t = dct32 ? dct32[(size_t)j * Mp + o] : (R)dct[(size_t)j * Mp + o];
                else t = dct[(size_t)j * Mp + o];
            }
            dcts[i] = t;
        }
        for (int jj = tid; jj < JC; jj += TPB) s2s[jj] = Samp::load_s2(sin2, min(j0 + jj, h));
        __syncthreads();
        // sample phase: this thread evaluates its own pair at jj = og, og+OG, ...
        const int jn = min(JC, h + 1 - j0);
#pragma unroll 2
        for (int jj = og; jj < JC; jj += OG)
            gsm[jj * PPB + pp] = (active && jj < jn) ? smp(s2s[jj]) : mk<R>(R(0), R(0));
        __syncthreads();
        if (!active) continue;
        const R *drow = dcts + og * NT;
        if constexpr (sizeof(R) == 4) {
            // FP32: 8-sample blocks folded into the running sums with Kahan
            // compensation (the node-level entries are double differences of
            // these orders, so their rounding must stay well below an ulp).
            // Packed f32x2 arithmetic on pairs of orders: acc[q] holds the real
            // parts of orders 2q, 2q + 1 and acc[NT/2 + q] their imaginary parts
            // (likewise cmp), so one instruction updates two orders.
            constexpr int H = NT / 2;
            for (int jb = 0; jb < jn; jb += 8) {
                float2 bR[H], bI[H];
#pragma unroll
                for (int q = 0; q < H; ++q) { bR[q] = make_float2(0.f, 0.f); bI[q] = bR[q]; }
                const int je = min(jb + 8, jn);
                for (int jj = jb; jj < je; ++jj) {
                    const CT gv = gsm[jj * PPB + pp];
                    const float2 gxx = make_float2(gv.x, gv.x), gyy = make_float2(gv.y, gv.y);
                    const float4 *row = reinterpret_cast<const float4 *>(drow + jj * NOB);
#pragma unroll
                    for (int n4 = 0; n4 < NT / 4; ++n4) {
                        const float4 c = row[n4];
                        const float2 c01 = make_float2(c.x, c.y), c23 = make_float2(c.z, c.w);
                        bR[2 * n4 + 0] = p2_fma(gxx, c01, bR[2 * n4 + 0]);
                        bI[2 * n4 + 0] = p2_fma(gyy, c01, bI[2 * n4 + 0]);
                        bR[2 * n4 + 1] = p2_fma(gxx, c23, bR[2 * n4 + 1]);
                        bI[2 * n4 + 1] = p2_fma(gyy, c23, bI[2 * n4 + 1]);
                    }
                }
#pragma unroll
                for (int q = 0; q < H; ++q) {
                    const float2 yr = p2_sub(bR[q], cmp[q]), yi = p2_sub(bI[q], cmp[H + q]);
                    const float2 tr = p2_add(acc[q], yr), ti = p2_add(acc[H + q], yi);
                    cmp[q] = p2_sub(p2_sub(tr, acc[q]), yr);
                    cmp[H + q] = p2_sub(p2_sub(ti, acc[H + q]), yi);
                    acc[q] = tr;
                    acc[H + q] = ti;
                }
            }
        } else {
            for (int jj = 0; jj < jn; ++jj) {
                const CT gv = gsm[jj * PPB + pp];
                const double2 *row = reinterpret_cast<const double2 *>(drow + jj * NOB);
#pragma unroll
                for (int n2 = 0; n2 < NT / 2; ++n2) {
                    const double2 c = row[n2];
                    acc[2 * n2 + 0].x = fma(gv.x, c.x, acc[2 * n2 + 0].x);
                    acc[2 * n2 + 0].y = fma(gv.y, c.x, acc[2 * n2 + 0].y);
                    acc[2 * n2 + 1].x = fma(gv.x, c.y, acc[2 * n2 + 1].x);
                    acc[2 * n2 + 1].y = fma(gv.y, c.y, acc[2 * n2 + 1].y);
                }
            }
        }
    }

    // per-pair orders to smem: FP32 path as double-float words (acc - cmp)
    if constexpr (sizeof(R) == 4) {
        float4 *Gf = reinterpret_cast<float4 *>(Gs);
        constexpr int H = NT / 2;
#pragma unroll
        for (int q = 0; q < H; ++q) {
            Gf[(ep * NOB + og * NT + 2 * q) * SLAB + gh] =
                make_float4(acc[q].x, -cmp[q].x, acc[H + q].x, -cmp[H + q].x);
            Gf[(ep * NOB + og * NT + 2 * q + 1) * SLAB + gh] =
                make_float4(acc[q].y, -cmp[q].y, acc[H + q].y, -cmp[H + q].y);
        }
    } else {
#pragma unroll
        for (int n = 0; n < NT; ++n)
            Gs[(ep * NOB + og * NT + n) * SLAB + gh] = make_double2(acc[n].x, acc[n].y);
    }
    __syncthreads();

    const double ik2 = 1.0 / (k * k);
    const float2 ik2f = df_from(ik2);
    // contraction: job (ep, n, b) = five order primitives of source node b for
    // both test nodes a.  Results replace the orders in place, so every
    // thread reads first and writes after a barrier (uniform trip count).
    const int njobs = EPB * nord * 2;
    for (int base = 0; base < njobs; base += TPB) {
        const int job = base + tid;
        const int jep = (job >> 1) / nord, n = (job >> 1) % nord, b = job & 1;
        const int ff = f0 + jep;
        const bool doit = job < njobs && ff < N && abs(e - ff) >= 2 && (!emask || emask[e] || emask[ff]);
        double2 out[5][2];    // p11, pdd, pds, psd, pss for a = 0, 1 (FP64 path)
        float4 outf[5][2];    // the same as double-float words (FP32 path)
        if (doit) {
            if constexpr (sizeof(R) == 4) {
                // double-float contraction (exact well below an FP32 ulp)
                const float4 *Gf = reinterpret_cast<const float4 *>(Gs) + (jep * NOB + n) * SLAB;
                const float2 *wt = wtf + EPB * 24;      // test element weights
                const float2 *ws = wtf + jep * 24;      // source element weights
                float4 GR1[4], GRs[4], GRd[4];          // (re.hi, re.lo, im.hi, im.lo) per g
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    float2 r1 = make_float2(0, 0), i1 = r1, rs = r1, is = r1, rd = r1, id = r1;
#pragma unroll
                    for (int hq = 0; hq < 4; ++hq) {
                        const float4 gv = Gf[g * 4 + hq];
                        const float2 gr = make_float2(gv.x, gv.y), gi = make_float2(gv.z, gv.w);
                        const float2 w1 = ws[(0 + b) * 4 + hq], wsv = ws[(2 + b) * 4 + hq], wd = ws[(4 + b) * 4 + hq];
                        df_mac(r1, gr, w1); df_mac(i1, gi, w1);
                        df_mac(rs, gr, wsv); df_mac(is, gi, wsv);
                        df_mac(rd, gr, wd); df_mac(id, gi, wd);
                    }
                    GR1[g] = make_float4(r1.x, r1.y, i1.x, i1.y);
                    GRs[g] = make_float4(rs.x, rs.y, is.x, is.y);
                    GRd[g] = make_float4(rd.x, rd.y, id.x, id.y);
                }
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    float2 acc2[5][2];
#pragma unroll
                    for (int c = 0; c < 5; ++c) { acc2[c][0] = make_float2(0, 0); acc2[c][1] = make_float2(0, 0); }
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        const float2 l1 = wt[(0 + a) * 4 + g], ls = wt[(2 + a) * 4 + g], ld = wt[(4 + a) * 4 + g];
                        const float4 q1 = GR1[g], qs = GRs[g], qd = GRd[g];
                        df_mac(acc2[0][0], l1, make_float2(q1.x, q1.y)); df_mac(acc2[0][1], l1, make_float2(q1.z, q1.w));
                        df_mac(acc2[1][0], ld, make_float2(qd.x, qd.y)); df_mac(acc2[1][1], ld, make_float2(qd.z, qd.w));
                        df_mac(acc2[2][0], ld, make_float2(qs.x, qs.y)); df_mac(acc2[2][1], ld, make_float2(qs.z, qs.w));
                        df_mac(acc2[3][0], ls, make_float2(qd.x, qd.y)); df_mac(acc2[3][1], ls, make_float2(qd.z, qd.w));
                        df_mac(acc2[4][0], ls, make_float2(qs.x, qs.y)); df_mac(acc2[4][1], ls, make_float2(qs.z, qs.w));
                    }
#pragma unroll
                    for (int c = 0; c < 5; ++c)
                        outf[c][a] = make_float4(acc2[c][0].x, acc2[c][0].y, acc2[c][1].x, acc2[c][1].y);
                }
            } else {
                const double2 *Gd = Gs + (jep * NOB + n) * SLAB;
                const double *wt = wts + EPB * 24;
                const double *ws = wts + jep * 24;
                double2 GR1[4], GRs[4], GRd[4];
#pragma unroll
                for (int g = 0; g < 4; ++g) {
                    double2 a1 = make_double2(0, 0), as = make_double2(0, 0), ad = make_double2(0, 0);
#pragma unroll
                    for (int hq = 0; hq < 4; ++hq) {
                        const double2 gv = Gd[g * 4 + hq];
                        const double w1 = ws[(0 + b) * 4 + hq], wsv = ws[(2 + b) * 4 + hq], wd = ws[(4 + b) * 4 + hq];
                        a1.x = fma(gv.x, w1, a1.x); a1.y = fma(gv.y, w1, a1.y);
                        as.x = fma(gv.x, wsv, as.x); as.y = fma(gv.y, wsv, as.y);
                        ad.x = fma(gv.x, wd, ad.x); ad.y = fma(gv.y, wd, ad.y);
                    }
                    GR1[g] = a1; GRs[g] = as; GRd[g] = ad;
                }
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    double2 q[5];
#pragma unroll
                    for (int c = 0; c < 5; ++c) q[c] = make_double2(0, 0);
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        const double l1 = wt[(0 + a) * 4 + g], ls = wt[(2 + a) * 4 + g], ld = wt[(4 + a) * 4 + g];
                        q[0].x = fma(l1, GR1[g].x, q[0].x); q[0].y = fma(l1, GR1[g].y, q[0].y);
                        q[1].x = fma(ld, GRd[g].x, q[1].x); q[1].y = fma(ld, GRd[g].y, q[1].y);
                        q[2].x = fma(ld, GRs[g].x, q[2].x); q[2].y = fma(ld, GRs[g].y, q[2].y);
                        q[3].x = fma(ls, GRd[g].x, q[3].x); q[3].y = fma(ls, GRd[g].y, q[3].y);
                        q[4].x = fma(ls, GRs[g].x, q[4].x); q[4].y = fma(ls, GRs[g].y, q[4].y);
                    }
#pragma unroll
                    for (int c = 0; c < 5; ++c) out[c][a] = q[c];
                }
            }
        }
        __syncthreads();      // every job of this pass has read its orders
        if constexpr (sizeof(R) == 4) {
            if (doit) {
                // mode-local parts in double-float (the FP64 pipe is ~1/64 of FP32)
                const int o = o0 + n;
                const float2 ttf = df_mul(df_from(geo[(size_t)10 * P + 4 * e]), df_from(geo[(size_t)10 * P + 4 * ff]));
                const float2 fmf = df_mulf(ik2f, (float)o), fm2f = df_mulf(fmf, (float)o);
                float4 *zl = reinterpret_cast<float4 *>(Gs + (jep * NOB + n) * SLAB);
                float4 *P11f = reinterpret_cast<float4 *>(P11s);
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const int ab = a * 2 + b;
                    const float4 p11 = outf[0][a], pdd = outf[1][a], pds = outf[2][a], psd = outf[3][a],
                                 pss = outf[4][a];
                    P11f[(jep * NOB + n) * 4 + ab] = p11;
                    zl[0 * 4 + ab] = f4(df_sub(df_mul(ttf, lo2(p11)), df_mul(ik2f, lo2(pdd))),
                                        df_sub(df_mul(ttf, hi2(p11)), df_mul(ik2f, hi2(pdd))));
                    zl[1 * 4 + ab] = f4(df_mul(fmf, hi2(pds)), df_neg(df_mul(fmf, lo2(pds))));   // -(j o/k^2) pds
                    zl[2 * 4 + ab] = f4(df_neg(df_mul(fmf, hi2(psd))), df_mul(fmf, lo2(psd)));   // +(j o/k^2) psd
                    zl[3 * 4 + ab] = f4(df_neg(df_mul(fm2f, lo2(pss))), df_neg(df_mul(fm2f, hi2(pss))));
                }
            }
        } else if (doit) {
            const int o = o0 + n;
            const double tze = geo[(size_t)10 * P + 4 * e], tzf = geo[(size_t)10 * P + 4 * ff];
            const double tt = tze * tzf;
            const double fm = o * ik2;               // jm/k^2 magnitude
            const double fm2 = (double)o * o * ik2;  // m^2/k^2
            double2 *zl = Gs + (jep * NOB + n) * SLAB;
            if constexpr (CK) {
                // the same parts with the complex 1/k^2
                double q[2];
                ck_inv_k2(k, ki, q);
                const double2 c1 = make_double2(q[0], q[1]);
                const double2 cm = make_double2(o * q[0], o * q[1]);
                const double2 cm2 = make_double2((double)o * o * q[0], (double)o * o * q[1]);
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const int ab = a * 2 + b;
                    const double2 p11 = out[0][a], pdd = out[1][a], pds = out[2][a], psd = out[3][a],
                                  pss = out[4][a];
                    P11s[(jep * NOB + n) * 4 + ab] = p11;
                    const double2 d = cmul(c1, pdd), x = cmul(cm, pds), y = cmul(cm, psd), w = cmul(cm2, pss);
                    zl[0 * 4 + ab] = make_double2(tt * p11.x - d.x, tt * p11.y - d.y);
                    zl[1 * 4 + ab] = make_double2(x.y, -x.x);                 // -(j o/k^2) pds
                    zl[2 * 4 + ab] = make_double2(-y.y, y.x);                 // +(j o/k^2) psd
                    zl[3 * 4 + ab] = make_double2(-w.x, -w.y);
                }
            } else {
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const int ab = a * 2 + b;
                    const double2 p11 = out[0][a], pdd = out[1][a], pds = out[2][a], psd = out[3][a],
                                  pss = out[4][a];
                    P11s[(jep * NOB + n) * 4 + ab] = p11;
                    // mode-local parts (mode m = o)
                    zl[0 * 4 + ab] = make_double2(tt * p11.x - ik2 * pdd.x, tt * p11.y - ik2 * pdd.y);
                    zl[1 * 4 + ab] = make_double2(fm * pds.y, -fm * pds.x);       // -(j o/k^2) pds
                    zl[2 * 4 + ab] = make_double2(-fm * psd.y, fm * psd.x);       // +(j o/k^2) psd
                    zl[3 * 4 + ab] = make_double2(-fm2 * pss.x, -fm2 * pss.y);
                }
            }
        }
        __syncthreads();
    }

    // mode combination + accumulation into Z[m]
    const int nmodes = m1 - m0 + 1;
    if constexpr (sizeof(R) == 4) {
        // double-float; each entry becomes a double only for its atomic add
        const float2 sre = df_from(sc_re), sim = df_from(sc_im);
        const float4 *P11f = reinterpret_cast<const float4 *>(P11s);
        for (int job = tid; job < EPB * nmodes; job += TPB) {
            const int jep = job / nmodes, m = m0 + job % nmodes;
            const int ff = f0 + jep;
            if (ff >= N || abs(e - ff) < 2 || (emask && !emask[e] && !emask[ff])) continue;
            const int nl = abs(m - 1) - o0, nm = m - o0, nh = m + 1 - o0;
            const float4 *zl = reinterpret_cast<const float4 *>(Gs + (jep * NOB + nm) * SLAB);
            const float2 tre = df_from(geo[(size_t)9 * P + 4 * e]), trf = df_from(geo[(size_t)9 * P + 4 * ff]);
            const float2 htt = df_mulf(df_mul(tre, trf), 0.5f), hre = df_mulf(tre, 0.5f), hrf = df_mulf(trf, 0.5f);
            double2 *Zm = Z + (size_t)m * mode_stride;
#pragma unroll
            for (int ab = 0; ab < 4; ++ab) {
                const int a = ab >> 1, b = ab & 1;
                const float4 lo = P11f[(jep * NOB + nl) * 4 + ab];
                const float4 hi = P11f[(jep * NOB + nh) * 4 + ab];
                const float2 Sr = df_add(lo2(lo), lo2(hi)), Si = df_add(hi2(lo), hi2(hi));
                const float2 Dr = df_sub(lo2(lo), lo2(hi)), Di = df_sub(hi2(lo), hi2(hi));
                float2 br[4], bi[4];
                const float4 z0 = zl[0 * 4 + ab], z1 = zl[1 * 4 + ab], z2 = zl[2 * 4 + ab], z3 = zl[3 * 4 + ab];
                br[0] = df_add(df_mul(htt, Sr), lo2(z0)); bi[0] = df_add(df_mul(htt, Si), hi2(z0));
                br[1] = df_add(df_mul(hre, Di), lo2(z1)); bi[1] = df_sub(hi2(z1), df_mul(hre, Dr));   // t_rho(e) D/(2j)
                br[2] = df_sub(lo2(z2), df_mul(hrf, Di)); bi[2] = df_add(df_mul(hrf, Dr), hi2(z2));   // -t_rho(f) D/(2j)
                br[3] = df_add(df_mulf(Sr, 0.5f), lo2(z3)); bi[3] = df_add(df_mulf(Si, 0.5f), hi2(z3));
                const long long r0 = e + a, c0 = ff + b;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const long long row = r0 + (q >> 1) * Nn, col = c0 + (q & 1) * Nn;
                    const float2 vr = df_sub(df_mul(sre, br[q]), df_mul(sim, bi[q]));
                    const float2 vi = df_add(df_mul(sre, bi[q]), df_mul(sim, br[q]));
                    catomic_add(Zm + row * ldz + col, make_double2(df_to_bits(vr), df_to_bits(vi)));
                }
            }
        }
    } else {
    for (int job = tid; job < EPB * nmodes; job += TPB) {
        const int jep = job / nmodes, m = m0 + job % nmodes;
        const int ff = f0 + jep;
        if (ff >= N || abs(e - ff) < 2 || (emask && !emask[e] && !emask[ff])) continue;
        const int nl = abs(m - 1) - o0, nm = m - o0, nh = m + 1 - o0;
        const double2 *zl = Gs + (jep * NOB + nm) * SLAB;
        const double tre = geo[(size_t)9 * P + 4 * e], trf = geo[(size_t)9 * P + 4 * ff];
        double2 *Zm = Z + (size_t)m * mode_stride;
#pragma unroll
        for (int ab = 0; ab < 4; ++ab) {
            const int a = ab >> 1, b = ab & 1;
            const double2 lo = P11s[(jep * NOB + nl) * 4 + ab];
            const double2 hi = P11s[(jep * NOB + nh) * 4 + ab];
            const double2 S = cadd(lo, hi), D = csub(lo, hi);
            double2 blk[4];
            blk[0] = cadd(make_double2(0.5 * tre * trf * S.x, 0.5 * tre * trf * S.y), zl[0 * 4 + ab]);
            blk[1] = cadd(make_double2(0.5 * tre * D.y, -0.5 * tre * D.x), zl[1 * 4 + ab]);   // t_rho(e) D/(2j)
            blk[2] = cadd(make_double2(-0.5 * trf * D.y, 0.5 * trf * D.x), zl[2 * 4 + ab]);   // -t_rho(f) D/(2j)
            blk[3] = cadd(make_double2(0.5 * S.x, 0.5 * S.y), zl[3 * 4 + ab]);
            const long long r0 = e + a, c0 = ff + b;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const long long row = r0 + (q >> 1) * Nn, col = c0 + (q & 1) * Nn;
                const double2 v = make_double2(sc_re * blk[q].x - sc_im * blk[q].y, sc_re * blk[q].y + sc_im * blk[q].x);
                catomic_add(Zm + row * ldz + col, v);
            }
        }
    }
    }
}

template <class R, int NT, int OG, bool CK = false>
int launch_far(int N, int M, int nxi, double k, double sre, double sim, const double *geo,
               const double *dct, const double *sin2, void *Z, long long ldz, long long ms,
               const unsigned char *emask, const float *dct32, cudaStream_t st, double ki = 0.0)
{
    constexpr int EPB = 16 / OG;
    const size_t smem = SmemLayout<R, NT, OG>::bytes();
    auto kern = far_efie_kernel<R, NT, OG, CK>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("far_efie: smem attribute");
    constexpr int NOB = OG * NT;
    const int fgroups = (N + EPB - 1) / EPB;
    const int nchunks = (M + 1 + (NOB - 2) - 1) / (NOB - 2);
    dim3 grid((unsigned)(N * fgroups), (unsigned)nchunks);
    kern<<<grid, TPB, smem, st>>>(N, N + 1, M, nxi / 2, k, sre, sim, geo, dct, sin2,
                                  reinterpret_cast<double2 *>(Z), ldz, ms, emask, dct32, ki);
    return check_launch(CK ? "far_efie (complex k)" : "far_efie");
}

}  // namespace
}  // namespace gb

extern "C" int ghost_bor_far_efie_masked(int prec, int n_elem, int m_max, int nxi, double k,
                                         double scale_re, double scale_im,
                                         const double *geo, const double *dct, const double *sin2,
                                         void *Z, long long ldz, long long mode_stride,
                                         const unsigned char *elem_mask, const float *dct32, void *stream)
{
    using namespace gb;
    if (n_elem < 3 || m_max < 0 || nxi < 2 || (nxi & 1) || !geo || !dct || !sin2 || !Z ||
        ldz < 2LL * (n_elem + 1) || mode_stride < ldz * 2LL * (n_elem + 1) || !(k > 0.0))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    // OG order groups x NT orders per thread: (8, 4) covers |m| <= 29 in one
    // launch row, (16, 4) |m| <= 61 and (16, 8) |m| <= 125 per row
    if (prec == GHOST_BOR_F32) {
        if (m_max + 1 <= 30) return launch_far<float, 8, 4>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, elem_mask, dct32, st);
        if (m_max + 1 <= 62) return launch_far<float, 16, 4>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, elem_mask, dct32, st);
        return launch_far<float, 16, 8>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, elem_mask, dct32, st);
    }
    if (prec == GHOST_BOR_F64) {
        if (m_max + 1 <= 30) return launch_far<double, 8, 4>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, elem_mask, dct32, st);
        return launch_far<double, 16, 4>(n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z, ldz, mode_stride, elem_mask, dct32, st);
    }
    return GHOST_BOR_EINVAL;
}

extern "C" int ghost_bor_far_efie(int prec, int n_elem, int m_max, int nxi, double k,
                                  double scale_re, double scale_im,
                                  const double *geo, const double *dct, const double *sin2,
                                  void *Z, long long ldz, long long mode_stride, void *stream)
{
    return ghost_bor_far_efie_masked(prec, n_elem, m_max, nxi, k, scale_re, scale_im, geo, dct, sin2, Z,
                                     ldz, mode_stride, nullptr, nullptr, stream);
}

extern "C" int ghost_bor_far_efie_ck(int n_elem, int m_max, int nxi, double k_re, double k_im,
                                     double scale_re, double scale_im,
                                     const double *geo, const double *dct, const double *sin2,
                                     void *Z, long long ldz, long long mode_stride, void *stream)
{
    using namespace gb;
    if (n_elem < 3 || m_max < 0 || nxi < 2 || (nxi & 1) || !geo || !dct || !sin2 || !Z ||
        ldz < 2LL * (n_elem + 1) || mode_stride < ldz * 2LL * (n_elem + 1) || !(k_re > 0.0) ||
        !(k_im <= 0.0) || !isfinite(k_re) || !isfinite(k_im))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (m_max + 1 <= 30)
        return launch_far<double, 8, 4, true>(n_elem, m_max, nxi, k_re, scale_re, scale_im, geo, dct, sin2, Z, ldz,
                                              mode_stride, nullptr, nullptr, st, k_im);
    return launch_far<double, 16, 4, true>(n_elem, m_max, nxi, k_re, scale_re, scale_im, geo, dct, sin2, Z, ldz,
                                           mode_stride, nullptr, nullptr, st, k_im);
}
