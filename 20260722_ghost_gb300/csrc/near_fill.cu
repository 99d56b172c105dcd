// near_fill.cu -- FP64 near/self EFIE element-pair blocks for all modes.
//
// Replaces the reference's refined near-pair path: graded cells
// (bor_solver.py:54-110), the near modal kernel (bor_kernels.py:170-257:
// sinh-graded core s in [0, s0] + Gauss tail xi in [xi0, pi]), and the near
// loop of assemble_mode (bor_solver.py:309-336).
//
// One CTA per element pair (e, f), |e - f| <= 1.  Threads own Gauss-point
// pairs of the graded cells; each evaluates G_n, n in a chunk of NC orders,
// by the two-piece azimuth quadrature with cos(n xi) from the Chebyshev
// recurrence (cos xi obtained from sin(xi/2) without an arcsine).  The CTA
// then contracts the pairs with the 20 Galerkin weights (5 primitives x 2x2
// nodes) as a small GEMM through shared memory, combines orders
// |m-1|, m, m+1 into the four mode-m blocks and adds scale * block into the
// output (FP64 band store or dense Z).
#include "common.cuh"

namespace gb {
namespace {

constexpr int TPBN = 128;      // point pairs per batch = threads
constexpr int NCORE = 48;      // sinh-core Gauss order (bor_kernels.py:170)
constexpr int kNc64 = 32;      // orders per chunk, FP64 projection
constexpr int kNcDf = 24;      // orders per chunk, double-float projection

struct NearSmem {
    // Gb   [TPBN][NC] double2 : per-pair orders of the current batch/chunk
    // W    [TPBN][20] double  : Galerkin weights of the batch
    // Prim [20][Mp]   double2 : contracted primitives, all orders
    static size_t bytes(int Mp, int NC) {
        return sizeof(double2) * (size_t)TPBN * NC + sizeof(double) * (size_t)TPBN * 20 +
               sizeof(double2) * 20 * (size_t)Mp;
    }
};

// acc[n] += (gre + j gim) cos((n0 + n) xi), n < NC, cos by the Chebyshev
// recurrence cos((n+1) xi) = 2 cos(xi) cos(n xi) - cos((n-1) xi).
template <bool DF, int NC>
__device__ __forceinline__ void project(double2 (&acc)[DF ? 1 : NC], float4 (&dacc)[DF ? NC : 1],
                                        double gre, double gim, double c1, int n0)
{
    if constexpr (!DF) {
        double cm1 = c1, c0 = 1.0;                  // cos(-xi), cos(0)
        for (int n = 0; n < n0; ++n) { const double cn = 2.0 * c1 * c0 - cm1; cm1 = c0; c0 = cn; }
#pragma unroll
        for (int n = 0; n < NC; ++n) {
            acc[n].x = fma(gre, c0, acc[n].x);
            acc[n].y = fma(gim, c0, acc[n].y);
            const double cn = 2.0 * c1 * c0 - cm1; cm1 = c0; c0 = cn;
        }
    } else {
        const float2 gr = df_from(gre), gi = df_from(gim);
        const float2 cf = df_from(c1);
        const float2 tc = make_float2(2.f * cf.x, 2.f * cf.y);   // exact doubling
        float2 cm1 = cf, c0 = make_float2(1.f, 0.f);
        for (int n = 0; n < n0; ++n) {
            const float2 cn = df_add(df_mul(tc, c0), make_float2(-cm1.x, -cm1.y));
            cm1 = c0; c0 = cn;
        }
#pragma unroll
        for (int n = 0; n < NC; ++n) {
            float2 ar = make_float2(dacc[n].x, dacc[n].y), ai = make_float2(dacc[n].z, dacc[n].w);
            df_mac(ar, gr, c0);
            df_mac(ai, gi, c0);
            dacc[n] = make_float4(ar.x, ar.y, ai.x, ai.y);
            const float2 cn = df_add(df_mul(tc, c0), make_float2(-cm1.x, -cm1.y));
            cm1 = c0; c0 = cn;
        }
    }
}

// DF = true: the cos(n xi) recurrence and the projection run in double-float
// (two FP32 words, ~48 bits) instead of FP64; the transcendental functions of
// each azimuth point stay FP64.
template <bool DF, int NC>
__global__ void __launch_bounds__(TPBN)
near_efie_kernel(int N, int Nn, int M, double k, double sc_re, double sc_im,
                 const double *__restrict__ nodes, const double *__restrict__ elem,
                 const int *__restrict__ pairs, const int *__restrict__ tails,
                 const double *__restrict__ cells, int ncells_total,
                 const double *__restrict__ core_gl, const double *__restrict__ tail_gl, int ntail_total,
                 double2 *__restrict__ band, double2 *__restrict__ Z, long long ldz, long long mode_stride)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Mp = M + 2;
    double2 *Gb = reinterpret_cast<double2 *>(smem_raw);
    double *W = reinterpret_cast<double *>(Gb + TPBN * NC);
    double2 *Prim = reinterpret_cast<double2 *>(W + TPBN * 20);

    const int pi = blockIdx.x;
    const int e = pairs[4 * pi + 0], f = pairs[4 * pi + 1];
    const int coff = pairs[4 * pi + 2], ncell = pairs[4 * pi + 3];
    const int toff = tails[2 * pi + 0], ntail = tails[2 * pi + 1];
    const int tid = threadIdx.x;

    const double rho_e0 = nodes[2 * e], z_e0 = nodes[2 * e + 1];
    const double drho_e = nodes[2 * e + 2] - rho_e0, dz_e = nodes[2 * e + 3] - z_e0;
    const double rho_f0 = nodes[2 * f], z_f0 = nodes[2 * f + 1];
    const double drho_f = nodes[2 * f + 2] - rho_f0, dz_f = nodes[2 * f + 3] - z_f0;
    const double Le = elem[e], Lf = elem[f];
    const double kk = k;

    for (int i = tid; i < 20 * Mp; i += TPBN) Prim[i] = make_double2(0.0, 0.0);

    const int nbatch = (ncell + TPBN - 1) / TPBN;
    const int nchunk = (Mp + NC - 1) / NC;
    for (int ch = 0; ch < nchunk; ++ch) {
        const int n0 = ch * NC;
        double2 out[(20 * NC + TPBN - 1) / TPBN];
#pragma unroll
        for (int r = 0; r < (20 * NC + TPBN - 1) / TPBN; ++r) out[r] = make_double2(0.0, 0.0);

        for (int bt = 0; bt < nbatch; ++bt) {
            const int c = bt * TPBN + tid;
            double2 acc[DF ? 1 : NC];   // FP64 projection
            float4 dacc[DF ? NC : 1];   // double-float projection: (re.hi, re.lo, im.hi, im.lo)
            double2 axis0 = make_double2(0.0, 0.0);   // order-0 term of an on-axis pair
            double wl[20];
#pragma unroll
            for (int n = 0; n < (DF ? 1 : NC); ++n) acc[n] = make_double2(0.0, 0.0);
#pragma unroll
            for (int n = 0; n < (DF ? NC : 1); ++n) dacc[n] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int i = 0; i < 20; ++i) wl[i] = 0.0;
            if (c < ncell) {
                const double s = cells[coff + c];
                const double sp = cells[ncells_total + coff + c];
                const double wc = cells[2 * ncells_total + coff + c];
                // points on the elements (bor_solver.py:117-127)
                const double rp = rho_e0 + s * drho_e, zp = z_e0 + s * dz_e;
                const double rq = rho_f0 + sp * drho_f, zq = z_f0 + sp * dz_f;
                const double w = wc * Le * Lf;
                // near modal kernel (bor_kernels.py:185-257)
                const double dr = rp - rq, dz = zp - zq;
                const double d2 = dr * dr + dz * dz;
                const double rr4 = 4.0 * rp * rq;
                if (rr4 <= 1e-30) {
                    if (n0 == 0) {
                        const double R0 = sqrt(d2);
                        double sn, cs;
                        sincos(kk * R0, &sn, &cs);
                        const double amp = 2.0 * GB_PI / (4.0 * GB_PI * fmax(R0, 1e-300));
                        axis0 = make_double2(amp * cs, -amp * sn);
                    }
                } else {
                    const double d = sqrt(fmax(d2, 1e-300));
                    const double a = sqrt(rr4);
                    const double da = d / a;
                    const double s0 = fmin(0.25, 20.0 * da);
                    const double vmax = asinh(s0 / da);
                    // -- sinh-graded core: s = (d/a) sinh(v), xi = 2 asin(s)
                    for (int i = 0; i < NCORE; ++i) {
                        const double v = core_gl[i] * vmax;
                        const double wv = core_gl[NCORE + i] * vmax;
                        const double sh = sinh(v), ch2 = cosh(v);
                        const double sv = fmin(da * sh, 1.0);
                        const double R = sqrt(d * d + (a * sv) * (a * sv));
                        const double dxi = 2.0 * da * ch2 / sqrt(fmax(1.0 - sv * sv, 1e-15));
                        double sn, cs;
                        sincos(kk * R, &sn, &cs);
                        const double gw = 2.0 * wv * dxi / (4.0 * GB_PI * R);
                        const double gre = gw * cs, gim = -gw * sn;
                        const double c1 = 1.0 - 2.0 * sv * sv;     // cos(xi)
                        project<DF, NC>(acc, dacc, gre, gim, c1, n0);
                    }
                    // -- Gauss tail on [xi0, pi]
                    const double xi0 = 2.0 * asin(s0);
                    const double span = GB_PI - xi0;
                    for (int i = 0; i < ntail; ++i) {
                        const double xi = xi0 + tail_gl[toff + i] * span;
                        const double wt = tail_gl[ntail_total + toff + i] * span;
                        double st, ct;
                        sincos(0.5 * xi, &st, &ct);
                        const double R = sqrt(d * d + (a * st) * (a * st));
                        double sn, cs;
                        sincos(kk * R, &sn, &cs);
                        const double gw = 2.0 * wt / (4.0 * GB_PI * R);
                        const double gre = gw * cs, gim = -gw * sn;
                        const double c1 = 1.0 - 2.0 * st * st;
                        project<DF, NC>(acc, dacc, gre, gim, c1, n0);
                    }
                }
                {
                    // Galerkin weights of this point pair (computed after the
                    // quadrature to keep them out of the registers it needs)
                    const double Tp[2] = {1.0 - s, s}, Tq[2] = {1.0 - sp, sp};
                    const double Dp[2] = {(drho_e * (1.0 - s) - rp) / Le, (drho_e * s + rp) / Le};
                    const double Dq[2] = {(drho_f * (1.0 - sp) - rq) / Lf, (drho_f * sp + rq) / Lf};
                    const double rr = rp * rq * w;
#pragma unroll
                    for (int a = 0; a < 2; ++a)
#pragma unroll
                        for (int b = 0; b < 2; ++b) {
                            const int ab = a * 2 + b;
                            wl[0 * 4 + ab] = Tp[a] * Tq[b] * rr;   // A1
                            wl[1 * 4 + ab] = Dp[a] * Dq[b] * w;    // Add
                            wl[2 * 4 + ab] = Dp[a] * Tq[b] * w;    // Ads
                            wl[3 * 4 + ab] = Tp[a] * Dq[b] * w;    // Asd
                            wl[4 * 4 + ab] = Tp[a] * Tq[b] * w;    // Ass
                        }
                }
            }
            __syncthreads();        // the previous batch's GEMM has finished reading W and Gb
            if constexpr (DF) {
#pragma unroll
                for (int n = 0; n < NC; ++n)
                    Gb[tid * NC + n] = make_double2((double)dacc[n].x + (double)dacc[n].y,
                                                    (double)dacc[n].z + (double)dacc[n].w);
            } else {
#pragma unroll
                for (int n = 0; n < NC; ++n) Gb[tid * NC + n] = acc[n];
            }
            if (n0 == 0) { Gb[tid * NC].x += axis0.x; Gb[tid * NC].y += axis0.y; }
#pragma unroll
            for (int i = 0; i < 20; ++i) W[tid * 20 + i] = wl[i];
            __syncthreads();
            // GEMM: out(c20, n) += sum_t W[t][c20] Gb[t][n]
            const int cnt = min(TPBN, ncell - bt * TPBN);
#pragma unroll
            for (int r = 0; r < (20 * NC + TPBN - 1) / TPBN; ++r) {
                const int o = tid + r * TPBN;
                if (o < 20 * NC) {
                    const int c20 = o / NC, n = o % NC;
                    double2 sacc = out[r];
                    for (int t = 0; t < cnt; ++t) {
                        const double wv = W[t * 20 + c20];
                        const double2 gv = Gb[t * NC + n];
                        sacc.x = fma(wv, gv.x, sacc.x);
                        sacc.y = fma(wv, gv.y, sacc.y);
                    }
                    out[r] = sacc;
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < (20 * NC + TPBN - 1) / TPBN; ++r) {
            const int o = tid + r * TPBN;
            if (o < 20 * NC) {
                const int c20 = o / NC, n = n0 + o % NC;
                if (n < Mp) Prim[c20 * Mp + n] = out[r];
            }
        }
        __syncthreads();
    }

    // mode combination: job = (m, blk, ab)
    const double ik2 = 1.0 / (kk * kk);
    const double tre = elem[N + e], tze = elem[2 * N + e];
    const double trf = elem[N + f], tzf = elem[2 * N + f];
    for (int job = tid; job < (M + 1) * 16; job += TPBN) {
        const int m = job / 16, blk = (job / 4) % 4, ab = job % 4;
        const int a = ab >> 1, b = ab & 1;
        const int ml = abs(m - 1), mh = m + 1;
        const double2 lo = Prim[(0 * 4 + ab) * Mp + ml], hi = Prim[(0 * 4 + ab) * Mp + mh];
        const double2 A1 = Prim[(0 * 4 + ab) * Mp + m];
        const double2 S = make_double2(0.5 * (lo.x + hi.x), 0.5 * (lo.y + hi.y));          // A1(Gc)
        const double2 Dh = make_double2(0.5 * (lo.x - hi.x), 0.5 * (lo.y - hi.y));         // (A1lo - A1hi)/2
        const double2 Gs = make_double2(Dh.y, -Dh.x);                                       // A1(Gs) = Dh / j
        const double fm = m * ik2, fm2 = (double)m * m * ik2;
        double2 v;
        if (blk == 0) {
            const double2 Add = Prim[(1 * 4 + ab) * Mp + m];
            v = make_double2(tre * trf * S.x + tze * tzf * A1.x - ik2 * Add.x,
                             tre * trf * S.y + tze * tzf * A1.y - ik2 * Add.y);
        } else if (blk == 1) {
            const double2 Ads = Prim[(2 * 4 + ab) * Mp + m];
            v = make_double2(tre * Gs.x + fm * Ads.y, tre * Gs.y - fm * Ads.x);
        } else if (blk == 2) {
            const double2 Asd = Prim[(3 * 4 + ab) * Mp + m];
            v = make_double2(-trf * Gs.x - fm * Asd.y, -trf * Gs.y + fm * Asd.x);
        } else {
            const double2 Ass = Prim[(4 * 4 + ab) * Mp + m];
            v = make_double2(S.x - fm2 * Ass.x, S.y - fm2 * Ass.y);
        }
        const double2 sv = make_double2(sc_re * v.x - sc_im * v.y, sc_re * v.y + sc_im * v.x);
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

}  // namespace
}  // namespace gb

extern "C" int ghost_bor_near_efie(int prec, int n_elem, int m_max, double k,
                                   double scale_re, double scale_im,
                                   const double *nodes, const double *elem,
                                   int n_pairs, const int *pairs, const int *tails,
                                   const double *cells, int n_cells_total,
                                   const double *core_gl, const double *tail_gl, int n_tail_total,
                                   double *band, void *Z, long long ldz, long long mode_stride,
                                   void *stream)
{
    using namespace gb;
    if (n_elem < 1 || m_max < 0 || n_pairs < 1 || !nodes || !elem || !pairs || !tails || !cells ||
        !core_gl || !tail_gl || !(k > 0.0))
        return GHOST_BOR_EINVAL;
    if (prec != GHOST_BOR_F32 && prec != GHOST_BOR_F64) return GHOST_BOR_EINVAL;
    if (!band && (!Z || ldz < 2LL * (n_elem + 1))) return GHOST_BOR_EINVAL;
    const bool df = prec == GHOST_BOR_F32;
    const size_t smem = NearSmem::bytes(m_max + 2, df ? kNcDf : kNc64);
    if (smem > 227 * 1024) return GHOST_BOR_EUNSUPPORTED;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    auto kern = df ? near_efie_kernel<true, kNcDf> : near_efie_kernel<false, kNc64>;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return check_launch("near_efie: smem attribute");
    kern<<<n_pairs, TPBN, smem, st>>>(
        n_elem, n_elem + 1, m_max, k, scale_re, scale_im, nodes, elem, pairs, tails, cells,
        n_cells_total, core_gl, tail_gl, n_tail_total, reinterpret_cast<double2 *>(band),
        reinterpret_cast<double2 *>(Z), ldz, mode_stride);
    return check_launch("near_efie");
}
