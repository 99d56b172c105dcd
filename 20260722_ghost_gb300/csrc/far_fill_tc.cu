// far_fill_tc.cu -- EFIE far fill with the azimuth transform on the bf16 tensor
// cores, exact to ~2^-30 of each Gauss-point pair's bound.
//
// Same result as far_fill.cu's FP32 path (the reference's streamed far
// assembly, bor_streaming.py:220-268, 320-376, 388-407, sampler
// bor_stream_kernel.c:26-48), with the even DCT
//
//     G_n = sum_j T[j][n] g_j,   j = 0..h  (h = n_xi / 2),  n = orders
//
// evaluated as a GEMM [64 point pairs x (re, im)] x [samples] x [orders] on
// tcgen05 instead of FP32 FMAs on the CUDA cores.  The FP32 table and the
// FP32 sums of the SIMT transform set its accuracy floor; here both operands
// are split into four balanced base-256 digits on a fixed-point grid
// (Ozaki's splitting):
//
//   row r (one point pair, re or im): g 2^(bA - e_r) = d0 + d1 2^-8 + d2 2^-16 + d3 2^-24
//   table:                            T 2^sT         = t0 + t1 2^-8 + t2 2^-16 + t3 2^-24
//
// with integer digits |d0| <= 2^bA, |t0| <= 128, |d1..d3|, |t1..t3| <= 128 (bf16
// holds them exactly, and every digit product exactly in FP32).  e_r is the
// analytic bound of the row, |g| = 1/R <= 1/|Delta| (R^2 = Delta^2 + 4 rho rho'
// sin^2(xi/2)); sT scales the table's largest entry to 128.  The samples come
// from a sampler ~50x more accurate than FP32 (TcGreen below) as two FP32
// words, and the digit split takes both.  The tensor core's FP32
// accumulation is not rounded to nearest, so each digit level s + t = L has
// an accumulator of its own, ACC_L, which adds integers only:
//   ACC0  (d0 t0): its sums stay below 2^24 (bA is chosen from the number of
//         samples K so that K 2^bA 128 <= 2^24): exact;
//   ACC1..ACC3: sums of 2..4 products per sample, random walks far below 2^24
//         (where one does reach it, its rounding is ~2^-32 of the row bound).
// The products with s + t > 3 are dropped (< 2^-32 of the row bound).  One
// accumulator for levels 1..3 costs ~60x in accuracy at 1025 samples (CPU
// emulation with truncating adds).  The epilogue forms
// ACC0 + 2^-8 ACC1 + 2^-16 ACC2 + 2^-24 ACC3 as a double-float and scales it.
//
// Kernel structure (one CTA per SM, persistent over tiles; a tile is one test
// element e x four source elements f0..f0+3, i.e. 64 Gauss-point pairs, for
// one range of orders):
//   warps 6..13  producers: sample g (TcGreen, FP32 word pairs) for 8
//                consecutive samples of one point pair, split them into the
//                four digit planes and store them into the A stage in the
//                UMMA K-major 64-byte-swizzled layout (32 samples per stage);
//   warp 4       TMA: the table digit planes of the stage (B operand);
//   warp 5       MMA: 10 tcgen05.mma kind::f16 per 16 samples into ACC0..3
//                (for tiles of up to 64 orders two TMEM accumulator sets, so a
//                tile's epilogue overlaps the next tile's transform; one set
//                of 4 x 128 columns for 128-order tiles);
//   warps 0..3   epilogue, warp w = element pair w: TMEM -> double-float
//                orders in shared memory (16 orders per chunk), then the
//                double-float contraction with the Galerkin weights, the
//                mode combination and the FP64 atomic accumulation into Z of
//                far_fill.cu.
// Every mbarrier wait is bounded; a wait that gives up sets the status word
// and the CTA drains its copies and MMAs before it frees TMEM and returns.
#include <cuda_bf16.h>

#include "common.cuh"
#include "df_math.cuh"
#include "samplers.cuh"
#include "tcgen05.cuh"

namespace gb {
namespace {

constexpr int TK = 32;               // samples per stage: 64-byte swizzled rows of bf16
constexpr int TM = 128;              // MMA rows: 4 element pairs x 16 point pairs x (re, im)
constexpr int ND = 4;                // digits per operand
constexpr int NEPI = 4;              // epilogue warps (TMEM lane quarters 0..3)
constexpr int W_TMA = 4, W_MMA = 5, W_PROD0 = 6;
constexpr int NPROD = 8;             // producer warps
constexpr int TC_THREADS = (W_PROD0 + NPROD) * 32;
constexpr int CH = 16;               // orders per epilogue chunk (one tcgen05.ld .x16 per accumulator)
constexpr int RING = CH + 2;         // order slabs per warp: a chunk plus the two carried orders
constexpr int SLAB = 17;             // float4 entries per order slab: 16 point pairs + 1 pad

template <int N> struct __align__(1024) TcSmem {
    __nv_bfloat16 a[2][ND][TM * TK];     // A stages: 128 rows x 64 B per digit plane
    __nv_bfloat16 b[2][ND][N * TK];      // B stages: N orders x 64 B per digit plane
    float4 g[NEPI][RING * SLAB];         // per-warp orders of its element pair (double-float)
    float4 zl[NEPI][RING * 2 * 16];      // per-warp mode-local blocks of every (order, orientation, block, a b)
    float4 p11[NEPI][RING * 2 * 4];      // per-warp 11-primitive of every (order, orientation, a b)
    float2 w[NEPI][2][24];               // test / source element weights (double-float)
    float4 sc_tab[kDfTabN];              // sin, cos (j pi / 128) as double-float words
    unsigned long long a_full[2], b_full[2], st_empty[2], t_full[2], t_empty[2], drain;
    uint32_t tmem_base;
    int failed;
};

// instruction descriptor: D f32, A/B bf16 (kind::f16), both K-major, M = 128, N
template <int N> constexpr uint32_t idesc_bf16()
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
}

// UMMA shared-memory descriptor: K-major operand, 64-byte swizzle, 8-row
// groups 512 bytes apart (SBO), version 1
__device__ __forceinline__ uint64_t umma_desc_sw64(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)((512u >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)4u << 61;             // SWIZZLE_64B
    return d;
}

template <int N>
__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                 ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc_bf16<N>()), "r"(accumulate));
}

// byte offset of (row r, 16-byte chunk c) in a K-major 64-byte-swizzled plane
__device__ __forceinline__ uint32_t sw64_off(int r, int c)
{
    return (uint32_t)((r >> 3) * 512 + (r & 7) * 64 + ((c ^ ((r >> 1) & 3)) << 4));
}

// exponent e of the row bound 1/|Delta| (|g| < 2^e for every sample of the pair)
__device__ __forceinline__ int row_exp(double d2)
{
    const double v = 1.0 / sqrt(d2) * (1.0 + 0x1p-12);
    return ilogb(v) + 1;
}

// Green's function samples g = exp(-j k R) / R (the 1/(4 pi) is in the table),
// each of re, im as an unnormalised pair hi + lo accurate to ~3e-9 of |g|
// (FP32 sincosf and rcp give ~1e-7, the floor of the FP32 fill):
//   R^2 = d^2 + a^2 s2 in double-float; R = r + rl and 1/R = y (1 + eps) from one
//   rsqrt and first-order corrections; k R in double-float, reduced to t in
//   [-pi, pi] by the three-word 2 pi of samplers.cuh;
//   sin and cos of t by Tang's table-driven method: t = j pi/128 + r,
//   |r| <= pi/256, with sin, cos (j pi/128) as double-float words (df_math.cuh
//   table), sin r = r - r^3/6 (next term < 2.5e-12) and
//   cos r - 1 = -r^2/2 + r^4/24 (next term < 5e-15); the table word carries the
//   value and one FP32 correction the rest, so the error is a few FP32
//   roundings of |correction| <= 0.013.
struct TcGreen {
    float d2h, d2l, a2h, a2l, kh, kl;
    __device__ void init(double d2, double a2, double k) {
        d2h = (float)d2; d2l = (float)(d2 - (double)d2h);
        a2h = (float)a2; a2l = (float)(a2 - (double)a2h);
        kh = (float)k;   kl = (float)(k - (double)kh);
    }
    // g as (re.hi, re.lo, im.hi, im.lo)
    __device__ __forceinline__ float4 operator()(float2 s2, const float4 *__restrict__ tab) const {
        const float p = a2h * s2.x;
        const float pe = fmaf(a2h, s2.x, -p);
        const float t = d2h + p;
        const float bb = t - d2h;
        const float te = (d2h - (t - bb)) + (p - bb);
        const float lo = te + pe + fmaf(a2h, s2.y, a2l * s2.x) + d2l;
        const float R2 = t + lo;
        const float R2l = lo - (R2 - t);
        const float y = rsqrtf(R2);
        const float r = R2 * y;
        const float rl = 0.5f * (fmaf(-r, r, R2) + R2l) * y;
        const float eps = fmaf(-r, y, 1.0f) - rl * y;        // 1/R = y (1 + eps)
        const float ph = kh * r;
        const float phl = fmaf(kh, r, -ph) + fmaf(kh, rl, kl * r);
        const float q = rintf(ph * kInvTwoPi);
        const float t1 = fmaf(-q, kTwoPiA, ph);             // exact
        const float qb = -q * kTwoPiB;                      // exact
        const float t2 = t1 + qb;
        const float tb = t2 - t1;
        const float t2e = (t1 - (t2 - tb)) + (qb - tb);
        const float dt = fmaf(-q, kTwoPiC, phl) + t2e;
        const float jf = fminf(128.0f, fmaxf(-128.0f, rintf(t2 * kDf128ByPi)));
        const float r0 = fmaf(-jf, kDfPiB128_1, t2);        // exact
        const float rv = fmaf(-jf, kDfPiB128_2, r0 + dt);
        const float r2 = rv * rv;
        const float sr = fmaf(rv * r2, -1.0f / 6.0f, rv);   // sin r
        const float c1 = r2 * fmaf(r2, 1.0f / 24.0f, -0.5f); // cos r - 1
        const float4 T = tab[(int)jf + 128];                 // sin hi, sin lo, cos hi, cos lo
        const float s_lo = fmaf(T.z, sr, fmaf(T.x, c1, T.y)) + T.w * sr;
        const float c_lo = fmaf(-T.x, sr, fmaf(T.z, c1, T.w)) - T.y * sr;
        const float yl = y * eps, ya = y + yl;
        const float gr = y * T.z;
        const float grl = fmaf(y, T.z, -gr) + fmaf(ya, c_lo, yl * T.z);
        const float gi = y * T.x;
        const float gil = fmaf(y, T.x, -gi) + fmaf(ya, s_lo, yl * T.x);
        return make_float4(gr, grl, -gi, -gil);
    }
};

__device__ __forceinline__ uint32_t pack_bf16(float2 d)
{
    const __nv_bfloat162 q = __floats2bfloat162_rn(d.x, d.y);
    return *reinterpret_cast<const uint32_t *>(&q);
}

// four balanced base-256 digits (integers, |d| <= 128) of two values hi + lo on
// the grid 2^(bA - e): packed FP32 pairs, rounding by the 1.5 * 2^23 shift.  The
// sampler's pairs are not normalised (|lo| reaches ~1% of |g|, and hi ~ 0 where
// the table's cosine or sine vanishes), so a two-sum normalises them first;
// the remainder after the top digit then takes the error word with one
// rounding (~2^-25 of a digit)
__device__ __forceinline__ void split4(float2 hi, float2 lo, float sc, uint32_t (&out)[ND])
{
    const float2 scv = make_float2(sc, sc), rn = make_float2(12582912.0f, 12582912.0f),
                 b256 = make_float2(256.0f, 256.0f);
    const float2 th = p2_mul(hi, scv), tl = p2_mul(lo, scv);
    float2 t = p2_add(th, tl);
    const float2 bb = p2_sub(t, th);
    const float2 te = p2_add(p2_sub(th, p2_sub(t, bb)), p2_sub(tl, bb));
    float2 d = p2_sub(p2_add(t, rn), rn);
    out[0] = pack_bf16(d);
    t = p2_add(p2_sub(t, d), te);
#pragma unroll
    for (int s = 1; s < ND; ++s) {
        t = p2_mul(t, b256);
        d = p2_sub(p2_add(t, rn), rn);
        out[s] = pack_bf16(d);
        t = p2_sub(t, d);
    }
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32"
                 " {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct TileGeo {
    int row, e, f0;
};

__device__ __forceinline__ TileGeo tile_of(long long t, int N, int fgroups)
{
    const long long per_row = (long long)N * fgroups;
    TileGeo g;
    g.row = (int)(t / per_row);
    const long long r = t % per_row;
    g.e = (int)(r / fgroups);
    g.f0 = (int)(r % fgroups) * 4;
    return g;
}

// far element pairs are visited once, as (e, f) with f >= e + 2; the mirror
// (f, e) reuses the same transform
__device__ __forceinline__ bool pair_active(int e, int f, int N) { return f < N && f >= e + 2; }
// a tile with at least one visited pair
__device__ __forceinline__ bool tile_live(const TileGeo &g, int N) { return g.f0 + 3 >= g.e + 2 && g.f0 < N; }

template <int N>
__global__ void __launch_bounds__(TC_THREADS, 1)
far_efie_tc_kernel(const __grid_constant__ CUtensorMap bmap, int NE, int Nn, int M, int h, double k,
                   double sc_re, double sc_im, const double *__restrict__ geo,
                   const float2 *__restrict__ s2f, const int *__restrict__ hdr, int bA,
                   double2 *__restrict__ Z, long long ldz, long long mode_stride, int *__restrict__ status)
{
    extern __shared__ unsigned char smem_raw[];
    TcSmem<N> &s = *reinterpret_cast<TcSmem<N> *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int P = 4 * NE;
    const int fgroups = (NE + 3) / 4;
    const int nrows = (M + 1 + (N - 2) - 1) / (N - 2);
    const long long ntiles = (long long)nrows * NE * fgroups;
    const int nst = (h + 1 + TK - 1) / TK;            // stages per tile
    constexpr int NSET = (8 * N <= 512) ? 2 : 1;       // accumulator sets (ACC0..ACC3) in TMEM
    constexpr uint32_t TMEM_COLS = (NSET * 4 * N <= 256) ? 256 : 512;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&s.tmem_base)), "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    df_fill_sincos_table(s.sc_tab);
    if (tid == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&s.a_full[i], NPROD);
            mbar_init(&s.b_full[i], 1);
            mbar_init(&s.st_empty[i], 1);
            mbar_init(&s.t_full[i], 1);
            mbar_init(&s.t_empty[i], NEPI);
        }
        mbar_init(&s.drain, 1);
        s.failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s.tmem_base;
    const int sT = hdr[1];
    volatile int *vfailed = &s.failed;
    auto fail = [&]() {
        *vfailed = 1;
        atomicExch(status, 1);
    };

    if (warp == W_TMA) {
        // ---------------- B operand: table digit planes, one stage per 32 samples
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)(ND * N * TK * 2);
            long long gs = 0;                                  // global stage counter
            for (long long t = blockIdx.x; t < ntiles && !*vfailed; t += gridDim.x) {
                const TileGeo tg = tile_of(t, NE, fgroups);
                if (!tile_live(tg, NE)) continue;
                const int o0 = max(0, tg.row * (N - 2) - 1);
                for (int ks = 0; ks < nst; ++ks, ++gs) {
                    const int st = (int)(gs & 1);
                    const long long use = gs >> 1;
                    if (use > 0 && !mbar_wait(&s.st_empty[st], (uint32_t)((use - 1) & 1))) { fail(); break; }
                    mbar_expect_tx(&s.b_full[st], bytes);
#pragma unroll
                    for (int q = 0; q < ND; ++q) tma_load_3d(s.b[st][q], &bmap, ks * TK, o0, q, &s.b_full[st]);
                }
            }
            // drain: every issued copy has landed before the CTA may exit
            for (int st = 0; st < 2; ++st) {
                const long long n_issued = (gs - st + 1) / 2;       // stages issued into slot st
                if (n_issued > 0 && !mbar_wait(&s.b_full[st], (uint32_t)((n_issued - 1) & 1))) fail();
            }
        }
    } else if (warp == W_MMA) {
        // ---------------- MMA issue
        if (lane == 0) {
            long long gs = 0, ti = 0;
            for (long long t = blockIdx.x; t < ntiles && !*vfailed; t += gridDim.x) {
                if (!tile_live(tile_of(t, NE, fgroups), NE)) continue;
                const int set = (int)(ti % NSET);
                const long long tuse = ti / NSET;
                ++ti;
                if (tuse > 0 && !mbar_wait(&s.t_empty[set], (uint32_t)((tuse - 1) & 1))) { fail(); break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc0 = tmem + (uint32_t)(set * 4 * N), acc1 = acc0 + N, acc2 = acc0 + 2 * N,
                               acc3 = acc0 + 3 * N;
                bool ok = true;
                for (int ks = 0; ks < nst; ++ks, ++gs) {
                    const int st = (int)(gs & 1);
                    const uint32_t par = (uint32_t)((gs >> 1) & 1);
                    if (!mbar_wait(&s.a_full[st], par) || !mbar_wait(&s.b_full[st], par)) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
                    for (int kk = 0; kk < TK / 16; ++kk) {
                        const uint32_t acc = (ks == 0 && kk == 0) ? 0u : 1u;
                        auto ad = [&](int q) { return umma_desc_sw64(smem_u32(s.a[st][q]) + kk * 32); };
                        auto bd = [&](int q) { return umma_desc_sw64(smem_u32(s.b[st][q]) + kk * 32); };
                        umma<N>(acc0, ad(0), bd(0), acc);
                        umma<N>(acc1, ad(0), bd(1), acc);
                        umma<N>(acc1, ad(1), bd(0), 1u);
                        umma<N>(acc2, ad(0), bd(2), acc);
                        umma<N>(acc2, ad(1), bd(1), 1u);
                        umma<N>(acc2, ad(2), bd(0), 1u);
                        umma<N>(acc3, ad(0), bd(3), acc);
                        umma<N>(acc3, ad(1), bd(2), 1u);
                        umma<N>(acc3, ad(2), bd(1), 1u);
                        umma<N>(acc3, ad(3), bd(0), 1u);
                    }
                    umma_commit(&s.st_empty[st]);
                }
                if (!ok) { fail(); break; }
                umma_commit(&s.t_full[set]);
            }
            // drain: every issued MMA has completed before TMEM is freed
            umma_commit(&s.drain);
            if (!mbar_wait(&s.drain, 0)) fail();
        }
    } else if (warp >= W_PROD0) {
        // ---------------- producers: samples -> digit planes of the A stage
        const int pt = tid - W_PROD0 * 32;
        const int ep = pt >> 6, jq = (pt >> 4) & 3, pp = pt & 15;
        const float2 *s2q = s2f + jq * 8;
        long long gs = 0;
        for (long long t = blockIdx.x; t < ntiles && !*vfailed; t += gridDim.x) {
            const TileGeo tg = tile_of(t, NE, fgroups);
            if (!tile_live(tg, NE)) continue;
            const int f = tg.f0 + ep;
            const bool act = pair_active(tg.e, f, NE);
            TcGreen smp;
            float sc = 0.f;
            if (act) {
                const int p = 4 * tg.e + (pp >> 2), q = 4 * f + (pp & 3);
                const double rp = geo[p], zp = geo[P + p], rq = geo[q], zq = geo[P + q];
                const double dr = rp - rq, dz = zp - zq;
                const double d2 = dr * dr + dz * dz;
                smp.init(d2, 4.0 * rp * rq, k);
                sc = ldexpf(1.0f, bA - row_exp(d2));
            }
            const int r_re = ep * 32 + pp, r_im = r_re + 16;
            for (int ks = 0; ks < nst; ++ks, ++gs) {
                const int st = (int)(gs & 1);
                const long long use = gs >> 1;
                if (use > 0 && !mbar_wait(&s.st_empty[st], (uint32_t)((use - 1) & 1))) { fail(); break; }
                if (act) {
                    const int j0 = ks * TK + jq * 8;
                    uint32_t wre[4][ND], wim[4][ND];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        float4 g0 = make_float4(0.f, 0.f, 0.f, 0.f), g1 = g0;
                        if (j0 + 2 * i <= h) g0 = smp(s2q[ks * TK + 2 * i], s.sc_tab);
                        if (j0 + 2 * i + 1 <= h) g1 = smp(s2q[ks * TK + 2 * i + 1], s.sc_tab);
                        split4(make_float2(g0.x, g1.x), make_float2(g0.y, g1.y), sc, wre[i]);
                        split4(make_float2(g0.z, g1.z), make_float2(g0.w, g1.w), sc, wim[i]);
                    }
                    unsigned char *abase = reinterpret_cast<unsigned char *>(s.a[st][0]);
#pragma unroll
                    for (int q = 0; q < ND; ++q) {
                        unsigned char *plane = abase + q * (TM * TK * 2);
                        *reinterpret_cast<uint4 *>(plane + sw64_off(r_re, jq)) =
                            make_uint4(wre[0][q], wre[1][q], wre[2][q], wre[3][q]);
                        *reinterpret_cast<uint4 *>(plane + sw64_off(r_im, jq)) =
                            make_uint4(wim[0][q], wim[1][q], wim[2][q], wim[3][q]);
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&s.a_full[st]);
            }
        }
    } else {
        // ---------------- epilogue: warp ep = element pair (e, f0 + ep) of the tile, and
        // its mirror (f0 + ep, e): g is symmetric in the point pair, so one transform
        // serves both orientations of the pair
        const int ep = warp;
        const int pp = lane & 15, cre = lane >> 4;           // row = ep*32 + cre*16 + pp
        float4 *G = s.g[ep];
        float4 *ZL = s.zl[ep];
        float4 *P11 = s.p11[ep];
        float2 *we = s.w[ep][0], *wf = s.w[ep][1];
        const double ik2 = 1.0 / (k * k);
        const float2 ik2f = df_from(ik2);
        const float2 sre = df_from(sc_re), sim = df_from(sc_im);
        long long ti = 0;
        for (long long t = blockIdx.x; t < ntiles && !*vfailed; t += gridDim.x) {
            const TileGeo tg = tile_of(t, NE, fgroups);
            if (!tile_live(tg, NE)) continue;
            const int e = tg.e, f = tg.f0 + ep;
            const bool act = pair_active(e, f, NE);
            const int m0 = tg.row * (N - 2);
            const int m1 = min(M, m0 + N - 3);
            const int o0 = max(0, m0 - 1);
            const int nord = m1 + 2 - o0;
            const int nch = (nord + CH - 1) / CH;
            const int set = (int)(ti % NSET);
            const uint32_t tpar = (uint32_t)((ti / NSET) & 1);
            ++ti;
            if (!mbar_wait(&s.t_full[set], tpar)) { fail(); break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            float scl = 0.f;
            float2 tre = make_float2(0.f, 0.f), trf = tre, ttf = tre;
            if (act) {
                if (lane < 24) {
                    we[lane] = df_from(geo[(size_t)(3 + lane / 4) * P + 4 * e + (lane % 4)]);
                    wf[lane] = df_from(geo[(size_t)(3 + lane / 4) * P + 4 * f + (lane % 4)]);
                }
                const int p = 4 * e + (pp >> 2), q = 4 * f + (pp & 3);
                const double dr = geo[p] - geo[q], dz = geo[P + p] - geo[P + q];
                scl = ldexpf(1.0f, row_exp(dr * dr + dz * dz) - bA - sT);
                tre = df_from(geo[(size_t)9 * P + 4 * e]);
                trf = df_from(geo[(size_t)9 * P + 4 * f]);
                ttf = df_mul(df_from(geo[(size_t)10 * P + 4 * e]), df_from(geo[(size_t)10 * P + 4 * f]));
            }
            __syncwarp();
            const uint32_t trow = tmem + ((uint32_t)(ep * 32) << 16) + (uint32_t)(set * 4 * N);
            for (int qc = 0; qc < nch; ++qc) {
                const int c_hi = min(CH, nord - qc * CH);      // orders of this chunk
                // (1) orders as double-float words, ACC0 + 2^-8 ACC1 (two-sum, exact) +
                //     2^-16 ACC2 + 2^-24 ACC3, times 2^(e_r - bA - sT)
                if (act) {
                    float a0[16], a1[16], a2[16], a3[16];
                    tmem_ld16(trow + (uint32_t)(qc * CH), a0);
                    tmem_ld16(trow + (uint32_t)(N + qc * CH), a1);
                    tmem_ld16(trow + (uint32_t)(2 * N + qc * CH), a2);
                    tmem_ld16(trow + (uint32_t)(3 * N + qc * CH), a3);
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        if (c < c_hi) {
                            const float x1 = a1[c] * 0x1p-8f;
                            const float sh = a0[c] + x1;
                            const float bb = sh - a0[c];
                            const float sl = (a0[c] - (sh - bb)) + (x1 - bb) + fmaf(a3[c], 0x1p-24f, a2[c] * 0x1p-16f);
                            const int slot = (qc * CH + c) % RING;
                            float2 *dst = reinterpret_cast<float2 *>(G + slot * SLAB + pp) + cre;
                            *dst = make_float2(sh * scl, sl * scl);
                        }
                    }
                }
                if (qc == nch - 1) {
                    // every TMEM read of this set is complete: release it to the MMA warp
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&s.t_empty[set]);
                }
                if (!act) continue;
                __syncwarp();
                // (2) contraction of both orientations: lane = (order, source node b);
                //     orientation 0 tests on e, sources on f; orientation 1 the mirror,
                //     whose point-pair orders are the transpose
                {
                    const int nl = qc * CH + (lane >> 1), b = lane & 1;
                    if ((lane >> 1) < c_hi) {
                        const int slot = nl % RING;
                        const float4 *Gf = G + slot * SLAB;
                        const int o = o0 + nl;
                        const float2 fmf = df_mulf(ik2f, (float)o), fm2f = df_mulf(fmf, (float)o);
#pragma unroll 1
                        for (int ori = 0; ori < 2; ++ori) {
                            const float2 *wt = ori ? wf : we, *ws = ori ? we : wf;
                            float4 GR1[4], GRs[4], GRd[4];
#pragma unroll
                            for (int g = 0; g < 4; ++g) {
                                float2 r1 = make_float2(0, 0), i1 = r1, rs = r1, is = r1, rd = r1, id = r1;
#pragma unroll
                                for (int hq = 0; hq < 4; ++hq) {
                                    const float4 gv = Gf[ori ? hq * 4 + g : g * 4 + hq];
                                    const float2 gr = make_float2(gv.x, gv.y), gi = make_float2(gv.z, gv.w);
                                    const float2 w1 = ws[(0 + b) * 4 + hq], wsv = ws[(2 + b) * 4 + hq],
                                                 wd = ws[(4 + b) * 4 + hq];
                                    df_mac(r1, gr, w1); df_mac(i1, gi, w1);
                                    df_mac(rs, gr, wsv); df_mac(is, gi, wsv);
                                    df_mac(rd, gr, wd); df_mac(id, gi, wd);
                                }
                                GR1[g] = make_float4(r1.x, r1.y, i1.x, i1.y);
                                GRs[g] = make_float4(rs.x, rs.y, is.x, is.y);
                                GRd[g] = make_float4(rd.x, rd.y, id.x, id.y);
                            }
                            float4 *zl = ZL + (slot * 2 + ori) * 16;
#pragma unroll 1
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
                                // p11, pdd, pds, psd, pss of test node a, source node b -> mode-local parts
                                const int ab = a * 2 + b;
                                const float2 p11r = acc2[0][0], p11i = acc2[0][1];
                                P11[(slot * 2 + ori) * 4 + ab] = make_float4(p11r.x, p11r.y, p11i.x, p11i.y);
                                zl[0 * 4 + ab] = f4(df_sub(df_mul(ttf, p11r), df_mul(ik2f, acc2[1][0])),
                                                    df_sub(df_mul(ttf, p11i), df_mul(ik2f, acc2[1][1])));
                                zl[1 * 4 + ab] = f4(df_mul(fmf, acc2[2][1]), df_neg(df_mul(fmf, acc2[2][0])));   // -(j o/k^2) pds
                                zl[2 * 4 + ab] = f4(df_neg(df_mul(fmf, acc2[3][1])), df_mul(fmf, acc2[3][0]));   // +(j o/k^2) psd
                                zl[3 * 4 + ab] = f4(df_neg(df_mul(fm2f, acc2[4][0])), df_neg(df_mul(fm2f, acc2[4][1])));
                            }
                        }
                    }
                }
                __syncwarp();
                // (3) modes whose orders |m-1|, m, m+1 are all in the ring now, both orientations
                const int mlo = (qc == 0) ? m0 : o0 + qc * CH - 1;
                const int mhi = min(m1, o0 + qc * CH + c_hi - 2);
                const int nm = mhi - mlo + 1;
                for (int job = lane; job < 8 * nm; job += 32) {
                    const int ori = job & 1, ab = (job >> 1) & 3, m = mlo + (job >> 3);
                    const int a = ab >> 1, b = ab & 1;
                    const float2 t_te = ori ? trf : tre, t_so = ori ? tre : trf;      // t_rho of test / source
                    const float2 htt = df_mulf(df_mul(t_te, t_so), 0.5f), hre = df_mulf(t_te, 0.5f),
                                 hrf = df_mulf(t_so, 0.5f);
                    const int sl = (abs(m - 1) - o0) % RING, sm = (m - o0) % RING, sh = (m + 1 - o0) % RING;
                    const float4 lo = P11[(sl * 2 + ori) * 4 + ab], hi = P11[(sh * 2 + ori) * 4 + ab];
                    const float4 *zl = ZL + (sm * 2 + ori) * 16;
                    const float2 Sr = df_add(lo2(lo), lo2(hi)), Si = df_add(hi2(lo), hi2(hi));
                    const float2 Dr = df_sub(lo2(lo), lo2(hi)), Di = df_sub(hi2(lo), hi2(hi));
                    float2 br[4], bi[4];
                    const float4 z0 = zl[0 * 4 + ab], z1 = zl[1 * 4 + ab], z2 = zl[2 * 4 + ab], z3 = zl[3 * 4 + ab];
                    br[0] = df_add(df_mul(htt, Sr), lo2(z0)); bi[0] = df_add(df_mul(htt, Si), hi2(z0));
                    br[1] = df_add(df_mul(hre, Di), lo2(z1)); bi[1] = df_sub(hi2(z1), df_mul(hre, Dr));
                    br[2] = df_sub(lo2(z2), df_mul(hrf, Di)); bi[2] = df_add(df_mul(hrf, Dr), hi2(z2));
                    br[3] = df_add(df_mulf(Sr, 0.5f), lo2(z3)); bi[3] = df_add(df_mulf(Si, 0.5f), hi2(z3));
                    double2 *Zm = Z + (size_t)m * mode_stride;
                    const long long r0 = (ori ? f : e) + a, c0 = (ori ? e : f) + b;
#pragma unroll
                    for (int qb = 0; qb < 4; ++qb) {
                        const long long row = r0 + (qb >> 1) * Nn, col = c0 + (qb & 1) * Nn;
                        const float2 vr = df_sub(df_mul(sre, br[qb]), df_mul(sim, bi[qb]));
                        const float2 vi = df_add(df_mul(sre, bi[qb]), df_mul(sim, br[qb]));
                        catomic_add(Zm + row * ldz + col, make_double2(df_to_bits(vr), df_to_bits(vi)));
                    }
                }
                __syncwarp();
            }
        }
    }

    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ---------------------------------------------------------------- tables
// header: [0] status, [1] sT; then s2f [Kpad] float2; then the digit planes
// bd [ND][Npad][Kpad] bf16 (orders as rows, samples contiguous)
__global__ void tc_table_scale_kernel(int h, int Mp, const double *__restrict__ dct, int *__restrict__ hdr)
{
    __shared__ double red[32];
    double m = 0.0;
    for (int i = threadIdx.x; i < (h + 1) * Mp; i += blockDim.x) m = fmax(m, fabs(dct[i]));
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
        // T 2^sT <= 128: the top digit is at most 128 in magnitude
        hdr[0] = 0;
        hdr[1] = (m > 0.0) ? 7 - ilogb(m) : 0;
    }
}

__global__ void tc_table_digits_kernel(int h, int Mp, int Npad, int Kpad, const double *__restrict__ dct,
                                       const double *__restrict__ sin2, const int *__restrict__ hdr,
                                       float2 *__restrict__ s2f, __nv_bfloat16 *__restrict__ bd)
{
    const int sT = hdr[1];
    const long long total = (long long)Npad * Kpad;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int o = (int)(i / Kpad), j = (int)(i % Kpad);
        double t = (o < Mp && j <= h) ? ldexp(dct[(size_t)j * Mp + o], sT) : 0.0;
#pragma unroll
        for (int s = 0; s < ND; ++s) {
            const double d = rint(t);
            bd[(size_t)s * total + i] = __float2bfloat16_rn((float)d);
            t = (t - d) * 256.0;
        }
        if (o == 0) {
            const double v = (j <= h) ? sin2[j] : 0.0;
            const float hi = (float)v;
            s2f[j] = make_float2(hi, (float)(v - (double)hi));
        }
    }
}

struct TcLayout {
    int N, Npad, Kpad;
    long long s2_off, bd_off, bytes;
};

TcLayout tc_layout(int m_max, int nxi)
{
    TcLayout L;
    const int Mp = m_max + 2;
    L.N = Mp <= 32 ? 32 : (Mp <= 64 ? 64 : 128);
    const int nrows = (m_max + 1 + (L.N - 2) - 1) / (L.N - 2);
    L.Npad = (nrows - 1) * (L.N - 2) + L.N;            // orders read by the last row's box
    const int h = nxi / 2;
    L.Kpad = ((h + 1 + TK - 1) / TK) * TK;
    L.s2_off = 256;
    L.bd_off = 256 + ((8LL * L.Kpad + 255) / 256) * 256;
    L.bytes = L.bd_off + 2LL * ND * L.Npad * L.Kpad;
    return L;
}

template <int N>
int launch_tc(const TcLayout &L, int NE, int M, int h, double k, double sre, double sim, const double *geo,
              unsigned char *w, int bA, double2 *Z, long long ldz, long long ms, cudaStream_t st)
{
    auto enc = get_encode();
    if (!enc) {
        set_last_error("far_efie_tc: cuTensorMapEncodeTiled unavailable");
        return GHOST_BOR_ECUDA;
    }
    CUtensorMap map;
    const cuuint64_t dims[3] = {(cuuint64_t)L.Kpad, (cuuint64_t)L.Npad, (cuuint64_t)ND};
    const cuuint64_t strides[2] = {(cuuint64_t)L.Kpad * 2, (cuuint64_t)L.Npad * L.Kpad * 2};
    const cuuint32_t box[3] = {TK, (cuuint32_t)N, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, w + L.bd_off, dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
        set_last_error("far_efie_tc: cuTensorMapEncodeTiled failed");
        return GHOST_BOR_ECUDA;
    }
    const size_t smem = sizeof(TcSmem<N>) + 1024;
    auto kern = far_efie_tc_kernel<N>;
    // once per process (and outside any stream capture: the first launch)
    static bool attr = false;
    static int nsm = 0;
    if (!attr) {
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return check_launch("far_efie_tc: smem attribute");
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
            nsm = 1;
        attr = true;
    }
    const int fgroups = (NE + 3) / 4;
    const int nrows = (M + 1 + (N - 2) - 1) / (N - 2);
    const long long ntiles = (long long)nrows * NE * fgroups;
    const int grid = (int)(ntiles < nsm ? ntiles : nsm);
    kern<<<grid, TC_THREADS, smem, st>>>(map, NE, NE + 1, M, h, k, sre, sim, geo,
                                         reinterpret_cast<const float2 *>(w + L.s2_off),
                                         reinterpret_cast<const int *>(w), bA, Z, ldz, ms,
                                         reinterpret_cast<int *>(w));
    return check_launch("far_efie_tc");
}

}  // namespace
}  // namespace gb

extern "C" long long ghost_bor_far_efie_tc_workspace(int m_max, int nxi)
{
    if (m_max < 0 || nxi < 2 || (nxi & 1)) return -1;
    return gb::tc_layout(m_max, nxi).bytes;
}

extern "C" int ghost_bor_far_efie_tc_tables(int m_max, int nxi, const double *dct, const double *sin2,
                                            void *work, long long work_bytes, void *stream)
{
    using namespace gb;
    if (m_max < 0 || nxi < 2 || (nxi & 1) || !dct || !sin2 || !work ||
        (reinterpret_cast<uintptr_t>(work) & 255) || work_bytes < ghost_bor_far_efie_tc_workspace(m_max, nxi))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const TcLayout L = tc_layout(m_max, nxi);
    unsigned char *w = reinterpret_cast<unsigned char *>(work);
    const int h = nxi / 2, Mp = m_max + 2;
    tc_table_scale_kernel<<<1, 1024, 0, st>>>(h, Mp, dct, reinterpret_cast<int *>(w));
    int rc = check_launch("far_efie_tc: table scale");
    if (rc) return rc;
    const long long total = (long long)L.Npad * L.Kpad;
    const int blocks = (int)((total + 255) / 256 < 4096 ? (total + 255) / 256 : 4096);
    tc_table_digits_kernel<<<blocks, 256, 0, st>>>(h, Mp, L.Npad, L.Kpad, dct, sin2, reinterpret_cast<const int *>(w),
                                                   reinterpret_cast<float2 *>(w + L.s2_off),
                                                   reinterpret_cast<__nv_bfloat16 *>(w + L.bd_off));
    return check_launch("far_efie_tc: table digits");
}

extern "C" int ghost_bor_far_efie_tc(int n_elem, int m_max, int nxi, double k, double scale_re, double scale_im,
                                     const double *geo, void *work, long long work_bytes,
                                     void *Z, long long ldz, long long mode_stride, void *stream)
{
    using namespace gb;
    if (n_elem < 3 || m_max < 0 || nxi < 2 || (nxi & 1) || !geo || !Z || !work ||
        (reinterpret_cast<uintptr_t>(work) & 255) || work_bytes < ghost_bor_far_efie_tc_workspace(m_max, nxi) ||
        ldz < 2LL * (n_elem + 1) || mode_stride < ldz * 2LL * (n_elem + 1) || !(k > 0.0))
        return GHOST_BOR_EINVAL;
    const int h = nxi / 2;
    // level-0 products d0 t0 (|d0| <= 2^bA, |t0| <= 128) summed over h + 1 samples stay below 2^24
    int bA = 7;
    while (bA > 1 && (long long)(h + 1) << (bA + 7) > (1LL << 24)) --bA;
    if ((long long)(h + 1) << (bA + 7) > (1LL << 24)) return GHOST_BOR_EUNSUPPORTED;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const TcLayout L = tc_layout(m_max, nxi);
    unsigned char *w = reinterpret_cast<unsigned char *>(work);
    double2 *Zd = reinterpret_cast<double2 *>(Z);
    if (L.N == 32) return launch_tc<32>(L, n_elem, m_max, h, k, scale_re, scale_im, geo, w, bA, Zd, ldz, mode_stride, st);
    if (L.N == 64) return launch_tc<64>(L, n_elem, m_max, h, k, scale_re, scale_im, geo, w, bA, Zd, ldz, mode_stride, st);
    return launch_tc<128>(L, n_elem, m_max, h, k, scale_re, scale_im, geo, w, bA, Zd, ldz, mode_stride, st);
}
