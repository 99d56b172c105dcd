// near_fill.cu -- FP64-class near/self EFIE element-pair blocks for all modes.
//
// Replaces the reference's refined near-pair path: graded cells
// (bor_solver.py:54-110), the near modal kernel (bor_kernels.py:170-257:
// sinh-graded core s in [0, s0] + Gauss tail xi in [xi0, pi]), and the near
// loop of assemble_mode (bor_solver.py:309-336).
//
// A persistent grid of CTAs walks the element pairs (e, f), |e - f| <= 1.
// Per batch of 128 Gauss-point pairs of the graded cells, each thread first
// evaluates its pair's azimuth nodes once -- g(xi) times the quadrature weight
// and cos(xi) -- into a per-CTA global scratch (node-major, so every access is
// coalesced); then, for each chunk of orders (NC, the remainder in chunks of
// 8), it projects the nodes onto cos(n xi) by the Chebyshev recurrence and the
// CTA contracts the pairs with the 20 Galerkin weights (5 primitives x 2x2
// nodes) as a small GEMM through shared memory.  The transcendental work is
// therefore done once per node instead of once per order chunk.  On the FP32
// path all of it runs in double-float arithmetic (df_math.cuh) on the FP32
// pipe, which on a GB300 is ~64x the FP64 pipe.
// Finally the CTA combines orders |m-1|, m, m+1 into the four mode-m blocks and
// adds scale * block into the output (FP64 band store or dense Z).
#include <type_traits>

#include "common.cuh"
#include "medium.cuh"
#include "df_math.cuh"

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
    // Tab  [257]     float4  : double-float sin, cos of j pi/128 (FP32 path)
    // Etab [32]      float2  : double-float 2^(j/32)
    // Core [2][48]   float2  : double-float sinh-core Gauss nodes and weights
    static size_t bytes(int Mp, int NC) {
        return sizeof(double2) * (size_t)TPBN * NC + sizeof(double) * (size_t)TPBN * 20 +
               sizeof(double2) * 20 * (size_t)Mp + sizeof(float4) * kDfTabN +
               sizeof(float2) * (kDfExpTabN + 2 * NCORE);
    }
};

// Per-node scratch of one CTA (node-major, [v][TPBN]): the weighted kernel
// value g w, cos(xi) and the Chebyshev state (cos((n-1) xi), cos(n xi)) at the
// start of the next order chunk.  DF: double-float words; FP64: doubles.
template <bool DF> struct NodeT;
template <> struct NodeT<true> { using A = float4; using B = float2; };
template <> struct NodeT<false> { using A = double2; using B = double; };
constexpr size_t kNodeBytes = 40;      // 16 + 3 * 8 per node and thread
// per-CTA double-float tail rule of the current pair (FP32 path): u, w and, for
// the standard tail (s0 = 1/4), sin^2(xi/2), w span / (2 pi), 1 - 2 sin^2(xi/2)
constexpr size_t kTailBytes = 5 * sizeof(float2);

// a node in double-float words: g w (complex) and cos(xi)
__device__ __forceinline__ void put_node_df(float4 *A, float2 *Bc, float2 *S0, float2 *S1, size_t i,
                                            float2 gre, float2 gim, float2 c1)
{
    A[i] = make_float4(gre.x, gre.y, gim.x, gim.y);
    Bc[i] = c1;
    S0[i] = c1;
    S1[i] = make_float2(1.f, 0.f);
}

__device__ __forceinline__ void put_node(double2 *A, double *Bc, double *S0, double *S1, size_t i,
                                         double gre, double gim, double c1)
{
    A[i] = make_double2(gre, gim);
    Bc[i] = c1;
    S0[i] = c1;
    S1[i] = 1.0;
}

// acc[n] += g cos((n0 + n) xi), n < NC, from the state (cm1, c0) =
// (cos((n0-1) xi), cos(n0 xi)) by the Chebyshev recurrence
// cos((n+1) xi) = 2 cos(xi) cos(n xi) - cos((n-1) xi); the state is advanced.
template <int NC>
__device__ __forceinline__ void project(double2 (&acc)[NC], double2 g, double c1, double &cm1, double &c0)
{
#pragma unroll
    for (int n = 0; n < NC; ++n) {
        acc[n].x = fma(g.x, c0, acc[n].x);
        acc[n].y = fma(g.y, c0, acc[n].y);
        const double cn = 2.0 * c1 * c0 - cm1; cm1 = c0; c0 = cn;
    }
}
template <int NC>
__device__ __forceinline__ void project(float4 (&dacc)[NC], float4 g, float2 cf, float2 &cm1, float2 &c0)
{
    // double-float order accumulators are kept as (re.hi, im.hi, re.lo, im.lo)
    // so that the packed f32x2 instructions of project2 work on (re, im) pairs
    const float2 gr = make_float2(g.x, g.y), gi = make_float2(g.z, g.w);
    const float2 tc = make_float2(2.f * cf.x, 2.f * cf.y);   // exact doubling
#pragma unroll
    for (int n = 0; n < NC; ++n) {
        float2 ar = make_float2(dacc[n].x, dacc[n].z), ai = make_float2(dacc[n].y, dacc[n].w);
        df_mac(ar, gr, c0);
        df_mac(ai, gi, c0);
        dacc[n] = make_float4(ar.x, ai.x, ar.y, ai.y);
        const float2 cn = df_add(df_mul(tc, c0), make_float2(-cm1.x, -cm1.y));
        cm1 = c0; c0 = cn;
    }
}

// Two nodes at once (double-float) on packed f32x2 instructions: the two
// recurrences run as the lanes of one pair (node a, node b), and each node's
// multiply-add into the (re, im) accumulators as the lanes of another; every
// rounding is that of df_mac / df_mul / df_add, so the result is the scalar one.
// S += G c with G = (re, im) of a node and c broadcast: Gh, Gl the high / low
// words of G, NGh = -Gh
__device__ __forceinline__ void p2_df_mac(float2 &Sh, float2 &Sl, float2 Gh, float2 Gl, float2 NGh, float2 Ch,
                                          float2 Cl)
{
    const float2 NP = p2_mul(NGh, Ch);                 // -p
    const float2 PE = p2_fma(Gh, Ch, NP);              // error of p
    const float2 T = p2_sub(Sh, NP);                   // s + p
    const float2 BB = p2_sub(T, Sh);
    const float2 TE = p2_sub(p2_sub(Sh, p2_sub(T, BB)), p2_add(NP, BB));
    const float2 X = p2_fma(Gh, Cl, p2_mul(Gl, Ch));
    Sl = p2_add(Sl, p2_add(p2_add(TE, PE), X));
    Sh = T;
}

template <int NC>
__device__ __forceinline__ void project2(float4 (&dacc)[NC], float4 g0, float2 cf0, float2 &cm0, float2 &cc0,
                                         float4 g1, float2 cf1, float2 &cm1, float2 &cc1)
{
    const float2 Gh0 = make_float2(g0.x, g0.z), Gl0 = make_float2(g0.y, g0.w), NGh0 = make_float2(-g0.x, -g0.z);
    const float2 Gh1 = make_float2(g1.x, g1.z), Gl1 = make_float2(g1.y, g1.w), NGh1 = make_float2(-g1.x, -g1.z);
    // recurrence lanes (node 0, node 1): t = 2 cos(xi), state (c_{n-1}, c_n)
    const float2 TCh = make_float2(2.f * cf0.x, 2.f * cf1.x), TCl = make_float2(2.f * cf0.y, 2.f * cf1.y);
    const float2 NTCh = make_float2(-TCh.x, -TCh.y);
    float2 CMh = make_float2(cm0.x, cm1.x), CMl = make_float2(cm0.y, cm1.y);
    float2 C0h = make_float2(cc0.x, cc1.x), C0l = make_float2(cc0.y, cc1.y);
#pragma unroll
    for (int n = 0; n < NC; ++n) {
        float2 Sh = make_float2(dacc[n].x, dacc[n].y), Sl = make_float2(dacc[n].z, dacc[n].w);
        p2_df_mac(Sh, Sl, Gh0, Gl0, NGh0, make_float2(C0h.x, C0h.x), make_float2(C0l.x, C0l.x));
        p2_df_mac(Sh, Sl, Gh1, Gl1, NGh1, make_float2(C0h.y, C0h.y), make_float2(C0l.y, C0l.y));
        dacc[n] = make_float4(Sh.x, Sh.y, Sl.x, Sl.y);
        // c_{n+1} = t c_n - c_{n-1}: df_mul then df_add, lane-wise
        const float2 NP = p2_mul(NTCh, C0h);
        float2 E = p2_fma(TCh, C0h, NP);
        E = p2_add(E, p2_fma(TCh, C0l, p2_mul(TCl, C0h)));
        const float2 H = p2_sub(E, NP);
        const float2 L = p2_sub(E, p2_add(H, NP));
        const float2 S = p2_sub(H, CMh);
        const float2 BB = p2_sub(S, H);
        float2 F = p2_sub(p2_sub(H, p2_sub(S, BB)), p2_add(CMh, BB));
        F = p2_sub(p2_add(F, L), CMl);
        const float2 Nh = p2_add(S, F);
        const float2 Nl = p2_sub(F, p2_sub(Nh, S));
        CMh = C0h; CMl = C0l;
        C0h = Nh; C0l = Nl;
    }
    cm0 = make_float2(CMh.x, CMl.x); cc0 = make_float2(C0h.x, C0l.x);
    cm1 = make_float2(CMh.y, CMl.y); cc1 = make_float2(C0h.y, C0l.y);
}

// per point pair constants of the double-float node evaluation
struct NodePairDF {
    float2 vmax, da, d2, a2, xi0, span;
    bool std_tail;                       // tail nodes tabulated (s0 = 1/4)
};

// double-float node v of a point pair (FP32 pipe): the weighted kernel value
// g w = (gre, gim) and cos(xi) (bor_kernels.py:185-257).  v < NCORE: the
// sinh-graded core, s = (d/a) sinh(t), xi = 2 asin(s); else the Gauss tail on
// [xi0, pi]
__device__ __forceinline__ void near_node_df(int v, const NodePairDF &P, const float2 *__restrict__ CoreX,
                                             const float2 *__restrict__ CoreW, const float2 *__restrict__ Etab,
                                             const float4 *__restrict__ Tab, const float2 *__restrict__ tU,
                                             const float2 *__restrict__ tWr, const float2 *__restrict__ tS2,
                                             const float2 *__restrict__ tWs, const float2 *__restrict__ tC1,
                                             float2 kf, float2 inv2pi, float2 &gre, float2 &gim, float2 &c1)
{
    const float2 one = make_float2(1.f, 0.f);
    float2 R2, gwn;
    if (v < NCORE) {
        // sinh and cosh from one e^t (and e^t - 1, exact for small t) and its reciprocal
        const float2 t = df_mul(CoreX[v], P.vmax);
        const float2 wv = df_mul(CoreW[v], P.vmax);
        float2 E, Em1;
        df_exp(t, Etab, E, Em1);
        const float2 iE = df_rcp(E);
        const float2 sh2 = df_mul(Em1, df_add(one, iE));        // 2 sinh t
        const float2 ch2 = df_add(E, iE);                        // 2 cosh t
        float2 sv = df_mul(P.da, make_float2(0.5f * sh2.x, 0.5f * sh2.y));
        if (sv.x >= 1.0f) sv = one;
        const float2 sv2 = df_mul(sv, sv);
        float2 om = df_add(one, make_float2(-sv2.x, -sv2.y));
        if (om.x < 1e-15f) om = make_float2(1e-15f, 0.f);
        // d xi / d t = 2 (d/a) cosh t / sqrt(1 - s^2)
        const float2 dxi = df_mul(df_mul(P.da, ch2), df_rsqrt(om));
        R2 = df_add(P.d2, df_mul(P.a2, sv2));
        gwn = df_mul(df_mul(wv, dxi), inv2pi);
        c1 = df_add(one, make_float2(-2.f * sv2.x, -2.f * sv2.y));
    } else {
        const int i = v - NCORE;
        float2 S2;
        if (P.std_tail) {
            S2 = tS2[i]; gwn = tWs[i]; c1 = tC1[i];
        } else {
            const float2 h2 = df_add(P.xi0, df_mul(tU[i], P.span));
            float2 sh, chh;
            df_sincos(make_float2(0.5f * h2.x, 0.5f * h2.y), Tab, sh, chh);
            S2 = df_mul(sh, sh);
            c1 = df_add(one, make_float2(-2.f * S2.x, -2.f * S2.y));
            gwn = df_mul(df_mul(tWr[i], P.span), inv2pi);
        }
        R2 = df_add(P.d2, df_mul(P.a2, S2));
    }
    const float2 iR = df_rsqrt(R2);
    const float2 R = df_mul(R2, iR);
    float2 sn, cs;
    df_sincos(df_reduce(df_mul(kf, R)), Tab, sn, cs);
    const float2 gw = df_mul(gwn, iR);
    gre = df_mul(gw, cs);
    const float2 gi = df_mul(gw, sn);
    gim = make_float2(-gi.x, -gi.y);
}

// one chunk of NCc orders n0 .. n0 + NCc - 1 for the current batch of point
// pairs: project every node of this thread's pair onto cos(n xi) (advancing
// the recurrence state in the scratch when more chunks follow), then contract
// the batch with the Galerkin weights into Prim
template <bool DF, int NCc>
__device__ __forceinline__ void near_chunk(int n0, bool more, bool valid, bool on_axis, double2 axis0, int nn,
                                           int tid, int cnt, int Mp, typename NodeT<DF>::A *gA,
                                           typename NodeT<DF>::B *gC, typename NodeT<DF>::B *gS0,
                                           typename NodeT<DF>::B *gS1, double2 *Gb, double *W, double2 *Prim)
{
    using NB = typename NodeT<DF>::B;
    using Acc = typename std::conditional<DF, float4, double2>::type;
    constexpr int NOUT = (20 * NCc + TPBN - 1) / TPBN;
    Acc acc[NCc];
#pragma unroll
    for (int n = 0; n < NCc; ++n) {
        if constexpr (DF) acc[n] = make_float4(0.f, 0.f, 0.f, 0.f);
        else acc[n] = make_double2(0.0, 0.0);
    }
    if (valid && !on_axis) {
        int v = 0;
        if constexpr (DF) {
            for (; v + 1 < nn; v += 2) {
                const size_t i = (size_t)v * TPBN + tid, j = i + TPBN;
                NB cma = gS0[i], c0a = gS1[i], cmb = gS0[j], c0b = gS1[j];
                project2<NCc>(acc, gA[i], gC[i], cma, c0a, gA[j], gC[j], cmb, c0b);
                if (more) { gS0[i] = cma; gS1[i] = c0a; gS0[j] = cmb; gS1[j] = c0b; }
            }
        }
        for (; v < nn; ++v) {
            const size_t i = (size_t)v * TPBN + tid;
            NB cm1 = gS0[i], c0 = gS1[i];
            project<NCc>(acc, gA[i], gC[i], cm1, c0);
            if (more) { gS0[i] = cm1; gS1[i] = c0; }
        }
    }
    __syncthreads();             // the previous chunk's GEMM has finished reading Gb
    if constexpr (DF) {
        // double-float orders and GEMM on the FP32 pipe
        float4 *Gf = reinterpret_cast<float4 *>(Gb);
#pragma unroll
        for (int n = 0; n < NCc; ++n) Gf[tid * NCc + n] = acc[n];
        if (n0 == 0 && on_axis) {
            const float2 ar = df_from(axis0.x), ai = df_from(axis0.y);
            Gf[tid * NCc] = make_float4(ar.x, ai.x, ar.y, ai.y);
        }
    } else {
#pragma unroll
        for (int n = 0; n < NCc; ++n) Gb[tid * NCc + n] = acc[n];
        if (n0 == 0) { Gb[tid * NCc].x += axis0.x; Gb[tid * NCc].y += axis0.y; }
    }
    __syncthreads();
    // GEMM: Prim(c20, n0 + n) += sum_t W[t][c20] Gb[t][n]; each (c20, n)
    // belongs to one thread, so the accumulation needs no atomics
#pragma unroll
    for (int r = 0; r < NOUT; ++r) {
        const int o = tid + r * TPBN;
        if (o < 20 * NCc) {
            const int c20 = o / NCc, n = o % NCc;
            double2 sacc;
            if constexpr (DF) {
                const float2 *Wf = reinterpret_cast<const float2 *>(W);
                const float4 *Gf = reinterpret_cast<const float4 *>(Gb);
                float2 sr = make_float2(0.f, 0.f), si = make_float2(0.f, 0.f);
                for (int t = 0; t < cnt; ++t) {
                    const float2 wv = Wf[t * 20 + c20];
                    const float4 gv = Gf[t * NCc + n];
                    df_mac(sr, wv, make_float2(gv.x, gv.z));
                    df_mac(si, wv, make_float2(gv.y, gv.w));
                }
                sacc = make_double2(df_to(sr), df_to(si));
            } else {
                sacc = make_double2(0.0, 0.0);
                for (int t = 0; t < cnt; ++t) {
                    const double wv = W[t * 20 + c20];
                    const double2 gv = Gb[t * NCc + n];
                    sacc.x = fma(wv, gv.x, sacc.x);
                    sacc.y = fma(wv, gv.y, sacc.y);
                }
            }
            if (n0 + n < Mp) {
                double2 &pr = Prim[c20 * Mp + n0 + n];
                pr.x += sacc.x;
                pr.y += sacc.y;
            }
        }
    }
}

// DF = true (FP32+IR path): every node's transcendental functions, the cos(m xi)
// recurrence, the projection and the order GEMM run in double-float (two FP32
// words, ~48 bits) on the FP32 pipe; DF = false is the plain FP64 path.
// CK: complex wave number k + j ki on the FP64 path (a lossy medium's
// interior): every sample of g gains e^{ki R}, and 1/k^2 is complex.
template <bool DF, int NC, bool CK = false>
__global__ void __launch_bounds__(TPBN, 2)
near_efie_kernel(int N, int Nn, int M, double k, double sc_re, double sc_im,
                 const double *__restrict__ nodes, const double *__restrict__ elem,
                 int n_pairs, const int *__restrict__ pairs, const int *__restrict__ tails,
                 const double *__restrict__ cells, int ncells_total,
                 const double *__restrict__ core_gl, const double *__restrict__ tail_gl, int ntail_total,
                 int nmax, double2 *__restrict__ band, double2 *__restrict__ Z, long long ldz,
                 long long mode_stride, unsigned char *__restrict__ scratch, int *__restrict__ status,
                 double ki)
{
    static_assert(!(CK && DF), "complex wave numbers on the FP64 path only");
    using NA = typename NodeT<DF>::A;
    using NB = typename NodeT<DF>::B;
    using Acc = typename std::conditional<DF, float4, double2>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Mp = M + 2;
    double2 *Gb = reinterpret_cast<double2 *>(smem_raw);
    double *W = reinterpret_cast<double *>(Gb + TPBN * NC);
    double2 *Prim = reinterpret_cast<double2 *>(W + TPBN * 20);
    float4 *Tab = reinterpret_cast<float4 *>(Prim + 20 * Mp);
    float2 *Etab = reinterpret_cast<float2 *>(Tab + kDfTabN);
    float2 *CoreX = Etab + kDfExpTabN, *CoreW = CoreX + NCORE;
    const int tid = threadIdx.x;

    const size_t plane = (size_t)nmax * TPBN;
    NA *gA = reinterpret_cast<NA *>(scratch + (size_t)blockIdx.x * plane * kNodeBytes);
    NB *gC = reinterpret_cast<NB *>(gA + plane);
    NB *gS0 = gC + plane;
    NB *gS1 = gS0 + plane;
    // double-float tail rule of the current pair (after every CTA's node planes)
    float2 *tU = reinterpret_cast<float2 *>(scratch + (size_t)gridDim.x * plane * kNodeBytes +
                                            (size_t)blockIdx.x * nmax * kTailBytes);
    float2 *tWr = tU + nmax, *tS2 = tWr + nmax, *tWs = tS2 + nmax, *tC1 = tWs + nmax;
    if constexpr (DF) {
        df_fill_sincos_table(Tab);
        df_fill_exp_table(Etab);
        for (int i = tid; i < NCORE; i += TPBN) {
            CoreX[i] = df_from(core_gl[i]);
            CoreW[i] = df_from(core_gl[NCORE + i]);
        }
    }
    const double span_std = GB_PI - 2.0 * asin(0.25);
    const float2 kf = df_from(k);
    const float2 inv2pi = df_from(1.0 / (2.0 * GB_PI));

    const double kk = k;

    for (int pi = blockIdx.x; pi < n_pairs; pi += gridDim.x) {
        const int e = pairs[4 * pi + 0], f = pairs[4 * pi + 1];
        const int coff = pairs[4 * pi + 2], ncell = pairs[4 * pi + 3];
        const int toff = tails[2 * pi + 0], ntail = tails[2 * pi + 1];
        const int nn = NCORE + ntail;
        if (nn > nmax) {                     // scratch sized for a smaller tail order
            if (tid == 0) atomicExch(status, 1);
            continue;
        }
        const double rho_e0 = nodes[2 * e], z_e0 = nodes[2 * e + 1];
        const double drho_e = nodes[2 * e + 2] - rho_e0, dz_e = nodes[2 * e + 3] - z_e0;
        const double rho_f0 = nodes[2 * f], z_f0 = nodes[2 * f + 1];
        const double drho_f = nodes[2 * f + 2] - rho_f0, dz_f = nodes[2 * f + 3] - z_f0;
        const double Le = elem[e], Lf = elem[f];

        __syncthreads();                     // the previous pair has finished reading Prim and its tail rule
        for (int i = tid; i < 20 * Mp; i += TPBN) Prim[i] = make_double2(0.0, 0.0);
        if constexpr (DF) {
            for (int i = tid; i < ntail; i += TPBN) {
                const double u = tail_gl[toff + i], w = tail_gl[ntail_total + toff + i];
                const double st = tail_gl[2 * ntail_total + toff + i];
                tU[i] = df_from(u);
                tWr[i] = df_from(w);
                tS2[i] = df_from(st * st);
                tWs[i] = df_from(w * span_std / (2.0 * GB_PI));
                tC1[i] = df_from(1.0 - 2.0 * st * st);
            }
            __syncthreads();
        }

        const int nbatch = (ncell + TPBN - 1) / TPBN;
        for (int bt = 0; bt < nbatch; ++bt) {
            const int c = bt * TPBN + tid;
            const bool valid = c < ncell;
            bool on_axis = false;
            double2 axis0 = make_double2(0.0, 0.0);   // order-0 term of an on-axis pair
            double wl[20];
#pragma unroll
            for (int i = 0; i < 20; ++i) wl[i] = 0.0;
            if (valid) {
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
                    on_axis = true;
                    const double R0 = sqrt(d2);
                    double sn, cs;
                    sincos(kk * R0, &sn, &cs);
                    double amp = 2.0 * GB_PI / (4.0 * GB_PI * fmax(R0, 1e-300));
                    if constexpr (CK) amp *= exp(ki * R0);
                    axis0 = make_double2(amp * cs, -amp * sn);
                } else {
                    const double d = sqrt(fmax(d2, 1e-300));
                    const double a = sqrt(rr4);
                    const double da = d / a;
                    const double s0 = fmin(0.25, 20.0 * da);
                    const double vmax = asinh(s0 / da);
                    // -- sinh-graded core: s = (d/a) sinh(v), xi = 2 asin(s)
                    const double xi0 = 2.0 * asin(s0);
                    const double span = GB_PI - xi0;
                    const bool std_tail = s0 == 0.25;          // tabulated half-angle nodes
                    if constexpr (DF) {
                        NodePairDF P;
                        P.vmax = df_from(vmax); P.da = df_from(da);
                        P.d2 = df_from(fmax(d2, 1e-300)); P.a2 = df_from(rr4);
                        P.xi0 = df_from(xi0); P.span = df_from(span); P.std_tail = std_tail;
#pragma unroll 1
                        for (int v = 0; v < nn; ++v) {
                            float2 gre, gim, c1;
                            near_node_df(v, P, CoreX, CoreW, Etab, Tab, tU, tWr, tS2, tWs, tC1, kf, inv2pi, gre,
                                         gim, c1);
                            put_node_df(gA, gC, gS0, gS1, (size_t)v * TPBN + tid, gre, gim, c1);
                        }
                    } else
                    for (int i = 0; i < NCORE; ++i) {
                        const double v = core_gl[i] * vmax;
                        const double wv = core_gl[NCORE + i] * vmax;
                        const double sh = sinh(v), ch2 = cosh(v);
                        const double sv = fmin(da * sh, 1.0);
                        // R and 1/R from one reciprocal square root
                        const double R2 = d * d + (a * sv) * (a * sv);
                        const double iR = rsqrt(R2);
                        const double R = R2 * iR;
                        const double dxi = 2.0 * da * ch2 * rsqrt(fmax(1.0 - sv * sv, 1e-15));
                        double sn, cs;
                        sincos(kk * R, &sn, &cs);
                        double gw = 2.0 * wv * dxi * (1.0 / (4.0 * GB_PI)) * iR;
                        if constexpr (CK) gw *= exp(ki * R);
                        put_node(gA, gC, gS0, gS1, (size_t)i * TPBN + tid, gw * cs, -gw * sn,
                                 1.0 - 2.0 * sv * sv);
                    }
                    // -- Gauss tail on [xi0, pi] (FP64 path)
                    if constexpr (!DF)
                    for (int i = 0; i < ntail; ++i) {
                        const double wt = tail_gl[ntail_total + toff + i] * span;
                        double st, ct;
                        if (std_tail) {
                            st = tail_gl[2 * ntail_total + toff + i];
                            ct = tail_gl[3 * ntail_total + toff + i];
                        } else {
                            sincos(0.5 * (xi0 + tail_gl[toff + i] * span), &st, &ct);
                        }
                        const double R2 = d * d + (a * st) * (a * st);
                        const double iR = rsqrt(R2);
                        const double R = R2 * iR;
                        double sn, cs;
                        sincos(kk * R, &sn, &cs);
                        double gw = 2.0 * wt * (1.0 / (4.0 * GB_PI)) * iR;
                        if constexpr (CK) gw *= exp(ki * R);
                        put_node(gA, gC, gS0, gS1, (size_t)(NCORE + i) * TPBN + tid, gw * cs, -gw * sn,
                                 1.0 - 2.0 * st * st);
                    }
                }
                // Galerkin weights of this point pair
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
            __syncthreads();                 // the previous batch's GEMM has finished reading W
            if constexpr (DF) {
                float2 *Wf = reinterpret_cast<float2 *>(W);
#pragma unroll
                for (int i = 0; i < 20; ++i) Wf[tid * 20 + i] = df_from(wl[i]);
            } else {
#pragma unroll
                for (int i = 0; i < 20; ++i) W[tid * 20 + i] = wl[i];
            }
            const int cnt = min(TPBN, ncell - bt * TPBN);

            // chunks of NC orders, then the remainder in chunks of 8 (or one more
            // full chunk when more than 16 orders remain)
            const int nfull = (Mp % NC > 16) ? (Mp + NC - 1) / NC : Mp / NC;
            const int ntl = nfull * NC >= Mp ? 0 : (Mp - nfull * NC + 7) / 8;
            for (int ch = 0; ch < nfull; ++ch)
                near_chunk<DF, NC>(ch * NC, ch + 1 < nfull || ntl > 0, valid, on_axis, axis0, nn, tid, cnt, Mp,
                                   gA, gC, gS0, gS1, Gb, W, Prim);
            for (int ch = 0; ch < ntl; ++ch)
                near_chunk<DF, 8>(nfull * NC + ch * 8, ch + 1 < ntl, valid, on_axis, axis0, nn, tid, cnt, Mp,
                                  gA, gC, gS0, gS1, Gb, W, Prim);
        }
        __syncthreads();

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
            if constexpr (CK) {
                // the same blocks with the complex 1/k^2: c1 = 1/k^2, cm = m/k^2, cm2 = m^2/k^2
                double q[2];
                ck_inv_k2(kk, ki, q);
                const double2 c1 = make_double2(q[0], q[1]);
                const double2 cm = make_double2(m * q[0], m * q[1]);
                const double2 cm2 = make_double2((double)m * m * q[0], (double)m * m * q[1]);
                if (blk == 0) {
                    const double2 d = cmul(c1, Prim[(1 * 4 + ab) * Mp + m]);
                    v = make_double2(tre * trf * S.x + tze * tzf * A1.x - d.x,
                                     tre * trf * S.y + tze * tzf * A1.y - d.y);
                } else if (blk == 1) {
                    const double2 x = cmul(cm, Prim[(2 * 4 + ab) * Mp + m]);
                    v = make_double2(tre * Gs.x + x.y, tre * Gs.y - x.x);       // - j (m/k^2) Ads
                } else if (blk == 2) {
                    const double2 y = cmul(cm, Prim[(3 * 4 + ab) * Mp + m]);
                    v = make_double2(-trf * Gs.x - y.y, -trf * Gs.y + y.x);     // + j (m/k^2) Asd
                } else {
                    const double2 w = cmul(cm2, Prim[(4 * 4 + ab) * Mp + m]);
                    v = make_double2(S.x - w.x, S.y - w.y);
                }
            } else if (blk == 0) {
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
}


// ---------------------------------------------------------------------------
// Grouped double-float near kernel (FP32+IR path): G lanes share one point
// pair.  Lane q of a group takes the orders n = q, q + G, q + 2G, ... (at most
// kOrdG) in registers, so one sweep over the azimuth nodes projects onto every
// order and no node data leaves the chip.  The group evaluates G nodes per
// round (one per lane), each lane also forming cos(k xi), k = 0..G, by the
// Chebyshev recurrence; the nodes go through shared memory, and lane q runs
// the step-G recurrence cos((n + G) xi) = 2 cos(G xi) cos(n xi) - cos((n - G) xi)
// from (cos((G - q) xi), cos(q xi)) over its orders.  The batch's orders are
// then contracted with the Galerkin weights into Prim and combined into the
// mode blocks as in near_efie_kernel.
// ---------------------------------------------------------------------------
constexpr int kOrdG = 16;      // orders per lane

// acc[i] += g c_i over the lane's orders, two nodes at a time on packed f32x2
// instructions (the rounding of df_mac / df_mul / df_add lane by lane): node
// a in lane .x, node b in lane .y of the recurrence pairs; t = 2 cos(G xi)
__device__ __forceinline__ void project_group2(float4 (&dacc)[kOrdG], int nord, float4 g0, float2 t0, float2 cm0,
                                               float2 cc0, float4 g1, float2 t1, float2 cm1, float2 cc1)
{
    const float2 Gh0 = make_float2(g0.x, g0.z), Gl0 = make_float2(g0.y, g0.w), NGh0 = make_float2(-g0.x, -g0.z);
    const float2 Gh1 = make_float2(g1.x, g1.z), Gl1 = make_float2(g1.y, g1.w), NGh1 = make_float2(-g1.x, -g1.z);
    const float2 TCh = make_float2(t0.x, t1.x), TCl = make_float2(t0.y, t1.y);
    const float2 NTCh = make_float2(-TCh.x, -TCh.y);
    float2 CMh = make_float2(cm0.x, cm1.x), CMl = make_float2(cm0.y, cm1.y);
    float2 C0h = make_float2(cc0.x, cc1.x), C0l = make_float2(cc0.y, cc1.y);
#pragma unroll
    for (int n = 0; n < kOrdG; ++n) {
        if (n >= nord) break;                  // uniform across the warp: no predicated tail
        {
            float2 Sh = make_float2(dacc[n].x, dacc[n].y), Sl = make_float2(dacc[n].z, dacc[n].w);
            p2_df_mac(Sh, Sl, Gh0, Gl0, NGh0, make_float2(C0h.x, C0h.x), make_float2(C0l.x, C0l.x));
            p2_df_mac(Sh, Sl, Gh1, Gl1, NGh1, make_float2(C0h.y, C0h.y), make_float2(C0l.y, C0l.y));
            dacc[n] = make_float4(Sh.x, Sh.y, Sl.x, Sl.y);
            const float2 NP = p2_mul(NTCh, C0h);
            float2 E = p2_fma(TCh, C0h, NP);
            E = p2_add(E, p2_fma(TCh, C0l, p2_mul(TCl, C0h)));
            const float2 H = p2_sub(E, NP);
            const float2 L = p2_sub(E, p2_add(H, NP));
            const float2 S = p2_sub(H, CMh);
            const float2 BB = p2_sub(S, H);
            float2 F = p2_sub(p2_sub(H, p2_sub(S, BB)), p2_add(CMh, BB));
            F = p2_sub(p2_add(F, L), CMl);
            const float2 Nh = p2_add(S, F);
            const float2 Nl = p2_sub(F, p2_sub(Nh, S));
            CMh = C0h; CMl = C0l;
            C0h = Nh; C0l = Nl;
        }
    }
}

struct NearGroupSmem {
    // Gb   [PPB][Mp]   float4 : orders of the batch's point pairs (double-float complex)
    // Prim [20][Mp]    double2: contracted primitives, all orders
    // W    [PPB][20]   float2 : double-float Galerkin weights of the batch
    // Xn   [TPBN][XN]  float  : exchanged nodes: g (4 words), cos(k xi) k = 0..G (2 words
    //                           each), padded to a multiple of 4 words (16-byte nodes)
    // Tab, Etab, CoreX, CoreW : double-float tables
    static size_t bytes(int G, int Mp) {
        const int PPB = TPBN / G, XN = (4 + 2 * (G + 1) + 3) / 4 * 4;
        return sizeof(float4) * (size_t)PPB * Mp + sizeof(double2) * 20 * (size_t)Mp + sizeof(float2) * PPB * 20 +
               sizeof(float) * (size_t)TPBN * XN + sizeof(float4) * kDfTabN +
               sizeof(float2) * (kDfExpTabN + 2 * NCORE);
    }
};

template <int G>
__global__ void __launch_bounds__(TPBN, 2)
near_efie_group_kernel(int N, int Nn, int M, double k, double sc_re, double sc_im,
                       const double *__restrict__ nodes, const double *__restrict__ elem,
                       int n_pairs, const int *__restrict__ pairs, const int *__restrict__ tails,
                       const double *__restrict__ cells, int ncells_total,
                       const double *__restrict__ core_gl, const double *__restrict__ tail_gl, int ntail_total,
                       int nmax, double2 *__restrict__ band, double2 *__restrict__ Z, long long ldz,
                       long long mode_stride, unsigned char *__restrict__ scratch, int *__restrict__ status)
{
    constexpr int PPB = TPBN / G;
    // floats per exchanged node, a multiple of 4 so that every node starts on 16 bytes
    constexpr int XN = (4 + 2 * (G + 1) + 3) / 4 * 4;
    static_assert(32 % G == 0 && G % 2 == 0, "a group of lanes lies in one warp");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Mp = M + 2;
    float4 *Gb = reinterpret_cast<float4 *>(smem_raw);
    double2 *Prim = reinterpret_cast<double2 *>(Gb + PPB * Mp);
    float2 *Wf = reinterpret_cast<float2 *>(Prim + 20 * Mp);
    float *Xn = reinterpret_cast<float *>(Wf + PPB * 20);
    float4 *Tab = reinterpret_cast<float4 *>(Xn + TPBN * XN);
    float2 *Etab = reinterpret_cast<float2 *>(Tab + kDfTabN);
    float2 *CoreX = Etab + kDfExpTabN, *CoreW = CoreX + NCORE;
    const int tid = threadIdx.x, grp = tid / G, q = tid % G;
    const int nord = (Mp + G - 1) / G;          // orders per lane (uniform; the last may pass Mp)

    // double-float tail rule of the current pair, per CTA
    float2 *tU = reinterpret_cast<float2 *>(scratch + (size_t)blockIdx.x * nmax * kTailBytes);
    float2 *tWr = tU + nmax, *tS2 = tWr + nmax, *tWs = tS2 + nmax, *tC1 = tWs + nmax;
    df_fill_sincos_table(Tab);
    df_fill_exp_table(Etab);
    for (int i = tid; i < NCORE; i += TPBN) {
        CoreX[i] = df_from(core_gl[i]);
        CoreW[i] = df_from(core_gl[NCORE + i]);
    }
    const double span_std = GB_PI - 2.0 * asin(0.25);
    const float2 kf = df_from(k);
    const float2 inv2pi = df_from(1.0 / (2.0 * GB_PI));

    for (int pi = blockIdx.x; pi < n_pairs; pi += gridDim.x) {
        const int e = pairs[4 * pi + 0], f = pairs[4 * pi + 1];
        const int coff = pairs[4 * pi + 2], ncell = pairs[4 * pi + 3];
        const int toff = tails[2 * pi + 0], ntail = tails[2 * pi + 1];
        const int nn = NCORE + ntail;
        if (nn > nmax) {                     // workspace sized for a smaller tail order
            if (tid == 0) atomicExch(status, 1);
            continue;
        }
        const double rho_e0 = nodes[2 * e], z_e0 = nodes[2 * e + 1];
        const double drho_e = nodes[2 * e + 2] - rho_e0, dz_e = nodes[2 * e + 3] - z_e0;
        const double rho_f0 = nodes[2 * f], z_f0 = nodes[2 * f + 1];
        const double drho_f = nodes[2 * f + 2] - rho_f0, dz_f = nodes[2 * f + 3] - z_f0;
        const double Le = elem[e], Lf = elem[f];

        __syncthreads();                     // the previous pair has finished reading Prim and its tail rule
        for (int i = tid; i < 20 * Mp; i += TPBN) Prim[i] = make_double2(0.0, 0.0);
        for (int i = tid; i < ntail; i += TPBN) {
            const double u = tail_gl[toff + i], w = tail_gl[ntail_total + toff + i];
            const double st = tail_gl[2 * ntail_total + toff + i];
            tU[i] = df_from(u);
            tWr[i] = df_from(w);
            tS2[i] = df_from(st * st);
            tWs[i] = df_from(w * span_std / (2.0 * GB_PI));
            tC1[i] = df_from(1.0 - 2.0 * st * st);
        }
        __syncthreads();

        const int nbatch = (ncell + PPB - 1) / PPB;
        for (int bt = 0; bt < nbatch; ++bt) {
            const int c = bt * PPB + grp;
            const bool valid = c < ncell;
            bool on_axis = false;
            double2 axis0 = make_double2(0.0, 0.0);
            NodePairDF P;
            double wl[20];
#pragma unroll
            for (int i = 0; i < 20; ++i) wl[i] = 0.0;
            if (valid) {
                const double s = cells[coff + c];
                const double sp = cells[ncells_total + coff + c];
                const double wc = cells[2 * ncells_total + coff + c];
                // points on the elements (bor_solver.py:117-127)
                const double rp = rho_e0 + s * drho_e, zp = z_e0 + s * dz_e;
                const double rq = rho_f0 + sp * drho_f, zq = z_f0 + sp * dz_f;
                const double w = wc * Le * Lf;
                const double dr = rp - rq, dz = zp - zq;
                const double d2 = dr * dr + dz * dz;
                const double rr4 = 4.0 * rp * rq;
                if (rr4 <= 1e-30) {
                    on_axis = true;
                    const double R0 = sqrt(d2);
                    double sn, cs;
                    sincos(k * R0, &sn, &cs);
                    const double amp = 2.0 * GB_PI / (4.0 * GB_PI * fmax(R0, 1e-300));
                    axis0 = make_double2(amp * cs, -amp * sn);
                } else {
                    const double d = sqrt(fmax(d2, 1e-300));
                    const double a = sqrt(rr4);
                    const double da = d / a;
                    const double s0 = fmin(0.25, 20.0 * da);
                    const double xi0 = 2.0 * asin(s0);
                    P.vmax = df_from(asinh(s0 / da));
                    P.da = df_from(da);
                    P.d2 = df_from(fmax(d2, 1e-300));
                    P.a2 = df_from(rr4);
                    P.xi0 = df_from(xi0);
                    P.span = df_from(GB_PI - xi0);
                    P.std_tail = s0 == 0.25;
                }
                // Galerkin weights of this point pair
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
            float4 acc[kOrdG];
#pragma unroll
            for (int i = 0; i < kOrdG; ++i) acc[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            // every lane of a group runs the same rounds (the group's pair decides)
            const bool nodes_on = valid && !on_axis;
            const int nround = nodes_on ? (nn + G - 1) / G : 0;
            float *xme = Xn + tid * XN;
            const float *xg = Xn + grp * G * XN;
            // the groups of a warp may run different numbers of rounds: sync the group only
            const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << ((tid & 31) & ~(G - 1));
            for (int r = 0; r < nround; ++r) {
                const int v = r * G + q;
                float2 gre = make_float2(0.f, 0.f), gim = gre, c1 = make_float2(1.f, 0.f);
                if (v < nn)
                    near_node_df(v, P, CoreX, CoreW, Etab, Tab, tU, tWr, tS2, tWs, tC1, kf, inv2pi, gre, gim, c1);
                // g and cos(k xi), k = 0..G (Chebyshev recurrence in double-float)
                reinterpret_cast<float4 *>(xme)[0] = make_float4(gre.x, gre.y, gim.x, gim.y);
                float2 *T = reinterpret_cast<float2 *>(xme + 4);
                const float2 tc = make_float2(2.f * c1.x, 2.f * c1.y);
                float2 tm = make_float2(1.f, 0.f), t0 = c1;
                T[0] = tm;
                T[1] = t0;
#pragma unroll
                for (int kk = 2; kk <= G; ++kk) {
                    const float2 tn = df_add(df_mul(tc, t0), make_float2(-tm.x, -tm.y));
                    T[kk] = tn;
                    tm = t0;
                    t0 = tn;
                }
                __syncwarp(gmask);
#pragma unroll 1
                for (int u = 0; u < G; u += 2) {
                    const float *xa = xg + u * XN, *xb = xa + XN;
                    const float4 ga = *reinterpret_cast<const float4 *>(xa);
                    const float4 gb = *reinterpret_cast<const float4 *>(xb);
                    const float2 *Ta = reinterpret_cast<const float2 *>(xa + 4);
                    const float2 *Tb = reinterpret_cast<const float2 *>(xb + 4);
                    const float2 ma = Ta[G], mb = Tb[G];
                    project_group2(acc, nord, ga, make_float2(2.f * ma.x, 2.f * ma.y), Ta[G - q], Ta[q], gb,
                                   make_float2(2.f * mb.x, 2.f * mb.y), Tb[G - q], Tb[q]);
                }
                __syncwarp(gmask);
            }
            if (valid && on_axis && q == 0) {
                const float2 ar = df_from(axis0.x), ai = df_from(axis0.y);
                acc[0] = make_float4(ar.x, ai.x, ar.y, ai.y);
            }
            __syncthreads();                 // the previous batch's GEMM has finished reading Gb and W
            if (q == 0) {
#pragma unroll
                for (int i = 0; i < 20; ++i) Wf[grp * 20 + i] = df_from(wl[i]);
            }
#pragma unroll
            for (int i = 0; i < kOrdG; ++i) {
                const int n = q + i * G;
                if (i < nord && n < Mp) Gb[grp * Mp + n] = acc[i];
            }
            __syncthreads();
            // GEMM: Prim(c20, n) += sum_t W[t][c20] Gb[t][n]; each (c20, n) belongs to one thread
            const int cnt = min(PPB, ncell - bt * PPB);
            for (int o = tid; o < 20 * Mp; o += TPBN) {
                const int c20 = o / Mp, n = o % Mp;
                float2 sr = make_float2(0.f, 0.f), si = make_float2(0.f, 0.f);
                for (int t = 0; t < cnt; ++t) {
                    const float2 wv = Wf[t * 20 + c20];
                    const float4 gv = Gb[t * Mp + n];
                    df_mac(sr, wv, make_float2(gv.x, gv.z));
                    df_mac(si, wv, make_float2(gv.y, gv.w));
                }
                double2 &pr = Prim[o];
                pr.x += df_to(sr);
                pr.y += df_to(si);
            }
        }
        __syncthreads();

        // mode combination: job = (m, blk, ab)
        const double ik2 = 1.0 / (k * k);
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
}

}  // namespace
}  // namespace gb

namespace gb {
// persistent grid of the near kernels: two CTAs per SM for the per-thread
// kernel and every resident CTA for the grouped one, unless set
int g_near_ctas_per_sm = 2;
int g_near_ctas_set = 0;

int near_grid()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
        sms = 1;
    return __atomic_load_n(&g_near_ctas_per_sm, __ATOMIC_RELAXED) * sms;
}
}  // namespace gb

extern "C" int ghost_bor_set_near_grid(int ctas_per_sm)
{
    if (ctas_per_sm < 0 || ctas_per_sm > 8) return GHOST_BOR_EINVAL;
    __atomic_store_n(&gb::g_near_ctas_per_sm, ctas_per_sm == 0 ? 2 : ctas_per_sm, __ATOMIC_RELAXED);
    __atomic_store_n(&gb::g_near_ctas_set, ctas_per_sm == 0 ? 0 : 1, __ATOMIC_RELAXED);
    return GHOST_BOR_OK;
}

extern "C" long long ghost_bor_near_workspace(int n_tail_max)
{
    if (n_tail_max < 0) return -1;
    return 256 + (long long)gb::near_grid() * (gb::NCORE + n_tail_max) *
                     ((long long)gb::TPBN * (long long)gb::kNodeBytes + (long long)gb::kTailBytes);
}

extern "C" int ghost_bor_near_efie(int prec, int n_elem, int m_max, double k,
                                   double scale_re, double scale_im,
                                   const double *nodes, const double *elem,
                                   int n_pairs, const int *pairs, const int *tails,
                                   const double *cells, int n_cells_total,
                                   const double *core_gl, const double *tail_gl, int n_tail_total,
                                   double *band, void *Z, long long ldz, long long mode_stride,
                                   int n_tail_max, void *work, long long work_bytes, void *stream)
{
    using namespace gb;
    if (n_elem < 1 || m_max < 0 || n_pairs < 1 || !nodes || !elem || !pairs || !tails || !cells ||
        !core_gl || !tail_gl || !(k > 0.0) || n_tail_max < 0 || !work ||
        (reinterpret_cast<uintptr_t>(work) & 255) || work_bytes < ghost_bor_near_workspace(n_tail_max))
        return GHOST_BOR_EINVAL;
    if (prec != GHOST_BOR_F32 && prec != GHOST_BOR_F64) return GHOST_BOR_EINVAL;
    if (!band && (!Z || ldz < 2LL * (n_elem + 1))) return GHOST_BOR_EINVAL;
    const bool df = prec == GHOST_BOR_F32;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int Mp = m_max + 2;
    // FP32+IR path: the grouped kernel, G lanes per point pair with at most kOrdG orders per lane
    // (the fewest lanes that hold the orders: fewer lanes per pair evaluate fewer
    // Chebyshev ladders and exchange fewer nodes)
    int gi = 0;
    while (gi < 4 && Mp > (2 << gi) * kOrdG) ++gi;
    const int G = gi < 4 ? (2 << gi) : 0;
    if (df && G) {
        const size_t gsm = NearGroupSmem::bytes(G, Mp);
        if (gsm > 227 * 1024) return GHOST_BOR_EUNSUPPORTED;
        decltype(&near_efie_group_kernel<2>) const kerns[4] = {near_efie_group_kernel<2>, near_efie_group_kernel<4>,
                                                               near_efie_group_kernel<8>, near_efie_group_kernel<16>};
        auto gk = kerns[gi];
        static bool gattr[4] = {false, false, false, false};
        if (!gattr[gi]) {
            if (cudaFuncSetAttribute(gk, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
                return check_launch("near_efie: smem attribute");
            gattr[gi] = true;
        }
        int *status = reinterpret_cast<int *>(work);
        if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return check_launch("near_efie: memset");
        // persistent grid: the resident CTAs of every SM (or the set number per SM)
        int dev = 0, sms = 1, occ = 1;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, gk, TPBN, gsm) != cudaSuccess || occ < 1)
            return check_launch("near_efie: occupancy");
        const int per_sm = __atomic_load_n(&g_near_ctas_set, __ATOMIC_RELAXED) ? near_grid() / sms : occ;
        const int gcap = sms * (per_sm < occ ? per_sm : occ);
        // the per-CTA tail rules fit the workspace of near_grid() CTAs' node planes
        if (256 + (long long)gcap * (NCORE + n_tail_max) * (long long)kTailBytes > work_bytes)
            return GHOST_BOR_EINVAL;
        const int grid = n_pairs < gcap ? n_pairs : gcap;
        gk<<<grid, TPBN, gsm, st>>>(
            n_elem, n_elem + 1, m_max, k, scale_re, scale_im, nodes, elem, n_pairs, pairs, tails, cells,
            n_cells_total, core_gl, tail_gl, n_tail_total, NCORE + n_tail_max,
            reinterpret_cast<double2 *>(band), reinterpret_cast<double2 *>(Z), ldz, mode_stride,
            reinterpret_cast<unsigned char *>(work) + 256, status);
        return check_launch("near_efie (grouped)");
    }
    const size_t smem = NearSmem::bytes(Mp, df ? kNcDf : kNc64);
    if (smem > 227 * 1024) return GHOST_BOR_EUNSUPPORTED;
    auto kern = df ? near_efie_kernel<true, kNcDf> : near_efie_kernel<false, kNc64>;
    // the largest dynamic shared memory, once per kernel (and before any
    // stream capture: the first launch); each launch asks for what it needs
    static bool attr[2] = {false, false};
    if (!attr[df ? 1 : 0]) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
            return check_launch("near_efie: smem attribute");
        attr[df ? 1 : 0] = true;
    }
    int *status = reinterpret_cast<int *>(work);
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return check_launch("near_efie: memset");
    const int grid = n_pairs < near_grid() ? n_pairs : near_grid();
    kern<<<grid, TPBN, smem, st>>>(
        n_elem, n_elem + 1, m_max, k, scale_re, scale_im, nodes, elem, n_pairs, pairs, tails, cells,
        n_cells_total, core_gl, tail_gl, n_tail_total, NCORE + n_tail_max,
        reinterpret_cast<double2 *>(band), reinterpret_cast<double2 *>(Z), ldz, mode_stride,
        reinterpret_cast<unsigned char *>(work) + 256, status, 0.0);
    return check_launch("near_efie");
}

extern "C" int ghost_bor_near_efie_ck(int n_elem, int m_max, double k_re, double k_im,
                                      double scale_re, double scale_im,
                                      const double *nodes, const double *elem,
                                      int n_pairs, const int *pairs, const int *tails,
                                      const double *cells, int n_cells_total,
                                      const double *core_gl, const double *tail_gl, int n_tail_total,
                                      double *band, void *Z, long long ldz, long long mode_stride,
                                      int n_tail_max, void *work, long long work_bytes, void *stream)
{
    using namespace gb;
    if (n_elem < 1 || m_max < 0 || n_pairs < 1 || !nodes || !elem || !pairs || !tails || !cells ||
        !core_gl || !tail_gl || !(k_re > 0.0) || !(k_im <= 0.0) || !isfinite(k_re) || !isfinite(k_im) ||
        n_tail_max < 0 || !work || (reinterpret_cast<uintptr_t>(work) & 255) ||
        work_bytes < ghost_bor_near_workspace(n_tail_max))
        return GHOST_BOR_EINVAL;
    if (!band && (!Z || ldz < 2LL * (n_elem + 1))) return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int Mp = m_max + 2;
    const size_t smem = NearSmem::bytes(Mp, kNc64);
    if (smem > 227 * 1024) return GHOST_BOR_EUNSUPPORTED;
    auto kern = near_efie_kernel<false, kNc64, true>;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) != cudaSuccess)
            return check_launch("near_efie_ck: smem attribute");
        attr = true;
    }
    int *status = reinterpret_cast<int *>(work);
    if (cudaMemsetAsync(status, 0, sizeof(int), st) != cudaSuccess) return check_launch("near_efie_ck: memset");
    const int grid = n_pairs < near_grid() ? n_pairs : near_grid();
    kern<<<grid, TPBN, smem, st>>>(
        n_elem, n_elem + 1, m_max, k_re, scale_re, scale_im, nodes, elem, n_pairs, pairs, tails, cells,
        n_cells_total, core_gl, tail_gl, n_tail_total, NCORE + n_tail_max,
        reinterpret_cast<double2 *>(band), reinterpret_cast<double2 *>(Z), ldz, mode_stride,
        reinterpret_cast<unsigned char *>(work) + 256, status, k_im);
    return check_launch("near_efie (complex k)");
}
