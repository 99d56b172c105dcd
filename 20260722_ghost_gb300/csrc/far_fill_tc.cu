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
// float4 entries per order slot of the mode-local blocks (4 blocks x 4 (a, b),
// + 2 pad) and of the 11-primitive (4 (a, b), + 6 pad): the pads put the 16
// orders of a chunk's lanes on distinct shared-memory banks
constexpr int ZLS = 18;
constexpr int P11S = 10;

template <int N> struct __align__(1024) TcSmem {
    __nv_bfloat16 a[2][ND][TM * TK];     // A stages: 128 rows x 64 B per digit plane
    __nv_bfloat16 b[2][ND][N * TK];      // B stages: N orders x 64 B per digit plane
    float4 g[NEPI][RING * SLAB];         // per-warp orders of its element pair (complex double-float)
    float4 zl[NEPI][RING * ZLS];         // per-warp mode-local blocks of every (order, block, a b)
    float4 p11[NEPI][RING * P11S];       // per-warp 11-primitive of every (order, a b)
    float2 w[NEPI][2][24];               // test / source element weights (double-float)
    float4 sc_tab[kDfTabN];              // sin, cos (j pi / 128) as double-float words
    unsigned long long a_full[2], b_full[2], st_empty[2], t_full[2], t_empty[2], drain;
    uint32_t tmem_base;
    int failed;
};

static_assert(sizeof(TcSmem<128>) + 1024 <= 227 * 1024, "TC far fill shared memory");

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

__device__ __forceinline__ float2 bcast(float x) { return make_float2(x, x); }

// |Delta|^2 = (rho_p - rho_q)^2 + (z_p - z_q)^2 of a point pair in double-float.
// Written with _rn intrinsics, which the compiler neither contracts nor
// reorders, so that the producers and the epilogue derive bit-identical row
// exponents from it
__device__ __forceinline__ float2 pair_d2(float2 rp, float2 zp, float2 rq, float2 zq)
{
    float2 d[2];
    const float2 a[2] = {rp, zp}, b[2] = {rq, zq};
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const float s = __fsub_rn(a[i].x, b[i].x);
        const float bb = __fsub_rn(s, a[i].x);
        const float e = __fadd_rn(__fadd_rn(__fsub_rn(a[i].x, __fsub_rn(s, bb)), __fsub_rn(-b[i].x, bb)),
                                  __fsub_rn(a[i].y, b[i].y));
        const float hh = __fadd_rn(s, e);
        d[i] = make_float2(hh, __fsub_rn(e, __fsub_rn(hh, s)));
    }
    float p[2], pe[2];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        p[i] = __fmul_rn(d[i].x, d[i].x);
        pe[i] = __fmaf_rn(__fmul_rn(2.0f, d[i].x), d[i].y, __fmaf_rn(d[i].x, d[i].x, -p[i]));
    }
    const float s = __fadd_rn(p[0], p[1]);
    const float bb = __fsub_rn(s, p[0]);
    const float e = __fadd_rn(__fadd_rn(__fsub_rn(p[0], __fsub_rn(s, bb)), __fsub_rn(p[1], bb)), __fadd_rn(pe[0], pe[1]));
    const float hh = __fadd_rn(s, e);
    return make_float2(hh, __fsub_rn(e, __fsub_rn(hh, s)));
}

// exponent e of the row bound 1/|Delta| (|g| < 2^e for every sample of the
// pair): the exponent field of rsqrt(|Delta|^2) (1 + 2^-10), the factor
// covering rsqrtf's and the sampler's relative errors (< 2^-20)
__device__ __forceinline__ int row_exp(float d2)
{
    const float v = __fmul_rn(rsqrtf(d2), 1.0f + 0x1p-10f);
    return ((__float_as_int(v) >> 23) & 0xff) - 126;
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
    __device__ void init(float2 d2, float2 a2, float2 k) {
        d2h = d2.x; d2l = d2.y;
        a2h = a2.x; a2l = a2.y;
        kh = k.x;   kl = k.y;
    }
    // g of two samples (sin^2 words s2h, s2l of samples A and B) with the f32x2
    // instructions: (re.hi, re.lo, im.hi, im.lo) each as an (A, B) pair.  The
    // negations -p, -r, ... are exact products with negated factors, so each
    // lane takes the same steps as the scalar formulas
    __device__ __forceinline__ void pair(float2 s2h, float2 s2l, const float4 *__restrict__ tab, float2 &gr,
                                         float2 &grl, float2 &gi, float2 &gil) const {
        const float2 A2H = bcast(a2h), D2H = bcast(d2h), KH = bcast(kh);
        const float2 pn = p2_mul(bcast(-a2h), s2h);                          // -p, p = a2h s2h
        const float2 pe = p2_fma(A2H, s2h, pn);
        const float2 t = p2_sub(D2H, pn);                                    // d2h + p
        const float2 bb = p2_sub(t, D2H);
        const float2 te = p2_sub(p2_sub(D2H, p2_sub(t, bb)), p2_add(pn, bb)); // (d2h - (t - bb)) + (p - bb)
        const float2 lo = p2_add(p2_add(p2_add(te, pe), p2_fma(A2H, s2l, p2_mul(bcast(a2l), s2h))), bcast(d2l));
        const float2 R2 = p2_add(t, lo);
        const float2 R2l = p2_sub(lo, p2_sub(R2, t));
        const float2 y = make_float2(rsqrtf(R2.x), rsqrtf(R2.y)), yn = make_float2(-y.x, -y.y);
        const float2 r = p2_mul(R2, y), rn = p2_mul(R2, yn);                 // r, -r
        const float2 rl = p2_mul(p2_mul(bcast(0.5f), p2_add(p2_fma(rn, r, R2), R2l)), y);
        const float2 eps = p2_sub(p2_fma(rn, y, bcast(1.0f)), p2_mul(rl, y));   // 1/R = y (1 + eps)
        const float2 ph = p2_mul(KH, r), phn = p2_mul(bcast(-kh), r);
        const float2 phl = p2_add(p2_fma(KH, r, phn), p2_fma(KH, rl, p2_mul(bcast(kl), r)));
        const float2 rn2 = bcast(12582912.0f);                               // 1.5 2^23: round to nearest even
        const float2 q = p2_sub(p2_add(p2_mul(ph, bcast(kInvTwoPi)), rn2), rn2);
        const float2 t1 = p2_fma(q, bcast(-kTwoPiA), ph);                    // exact
        const float2 qb = p2_mul(q, bcast(-kTwoPiB));                        // exact
        const float2 t2 = p2_add(t1, qb);
        const float2 tb = p2_sub(t2, t1);
        const float2 t2e = p2_add(p2_sub(t1, p2_sub(t2, tb)), p2_sub(qb, tb));
        const float2 dt = p2_add(p2_fma(q, bcast(-kTwoPiC), phl), t2e);
        float2 jf = p2_sub(p2_add(p2_mul(t2, bcast(kDf128ByPi)), rn2), rn2);
        jf = make_float2(fminf(128.0f, fmaxf(-128.0f, jf.x)), fminf(128.0f, fmaxf(-128.0f, jf.y)));
        const float2 r0 = p2_fma(jf, bcast(-kDfPiB128_1), t2);               // exact
        const float2 rv = p2_fma(jf, bcast(-kDfPiB128_2), p2_add(r0, dt));
        const float2 r2 = p2_mul(rv, rv);
        const float2 sr = p2_fma(p2_mul(rv, r2), bcast(-1.0f / 6.0f), rv);  // sin r
        const float2 c1 = p2_mul(r2, p2_fma(r2, bcast(1.0f / 24.0f), bcast(-0.5f)));   // cos r - 1
        const float4 TA = tab[(int)jf.x + 128], TB = tab[(int)jf.y + 128];  // sin hi, sin lo, cos hi, cos lo
        const float2 Sh = make_float2(TA.x, TB.x), Sl = make_float2(TA.y, TB.y), Ch = make_float2(TA.z, TB.z),
                     Cl = make_float2(TA.w, TB.w), Shn = make_float2(-TA.x, -TB.x);
        const float2 s_lo = p2_add(p2_fma(Ch, sr, p2_fma(Sh, c1, Sl)), p2_mul(Cl, sr));
        const float2 c_lo = p2_sub(p2_fma(Shn, sr, p2_fma(Ch, c1, Cl)), p2_mul(Sl, sr));
        const float2 yl = p2_mul(y, eps), ya = p2_add(y, yl);
        gr = p2_mul(y, Ch);
        grl = p2_add(p2_fma(y, Ch, p2_mul(yn, Ch)), p2_fma(ya, c_lo, p2_mul(yl, Ch)));
        // the imaginary part -y sin: returned as +y sin, the caller negates its digit scale
        gi = p2_mul(y, Sh);
        gil = p2_add(p2_fma(y, Sh, p2_mul(yn, Sh)), p2_fma(ya, s_lo, p2_mul(yl, Sh)));
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

// complex double-float with its parts packed for the f32x2 instructions:
// h = (re.hi, im.hi), l = (re.lo, im.lo), so that one packed instruction takes
// the same step for the real and the imaginary part.  In shared memory as a
// float4 (re.hi, im.hi, re.lo, im.lo)
struct cdf {
    float2 h, l;
};
__device__ __forceinline__ cdf cdf_of(float4 v) { return {make_float2(v.x, v.y), make_float2(v.z, v.w)}; }
__device__ __forceinline__ float4 cdf_f4(const cdf &a) { return make_float4(a.h.x, a.h.y, a.l.x, a.l.y); }
__device__ __forceinline__ cdf cdf_zero() { return {make_float2(0.f, 0.f), make_float2(0.f, 0.f)}; }
__device__ __forceinline__ cdf cdf_neg(const cdf &a) { return {make_float2(-a.h.x, -a.h.y), make_float2(-a.l.x, -a.l.y)}; }
__device__ __forceinline__ cdf cdf_j(const cdf &a) { return {make_float2(-a.h.y, a.h.x), make_float2(-a.l.y, a.l.x)}; }
__device__ __forceinline__ cdf cdf_mj(const cdf &a) { return {make_float2(a.h.y, -a.h.x), make_float2(a.l.y, -a.l.x)}; }
__device__ __forceinline__ cdf cdf_half(const cdf &a) { return {p2_mul(a.h, bcast(0.5f)), p2_mul(a.l, bcast(0.5f))}; }

// s += a w with w a real double-float (df_mac on both parts); s.l is left
// unnormalised, |s.l| << |s.h|
__device__ __forceinline__ void cdf_mac(cdf &s, const cdf &a, float2 w)
{
    const float2 W = bcast(w.x);
    const float2 pn = p2_mul(a.h, bcast(-w.x));                              // -p, p = a.h w.hi
    const float2 pe = p2_fma(a.h, W, pn);                                    // a.h w.hi - p, exact
    const float2 t = p2_sub(s.h, pn);                                        // s.h + p
    const float2 bb = p2_sub(t, s.h);
    const float2 te = p2_sub(p2_sub(s.h, p2_sub(t, bb)), p2_add(pn, bb));    // two-sum error
    const float2 cr = p2_fma(a.h, bcast(w.y), p2_mul(a.l, W));
    s.l = p2_add(s.l, p2_add(p2_add(te, pe), cr));
    s.h = t;
}
// a w with w a real double-float, renormalised (df_mul on both parts)
__device__ __forceinline__ cdf cdf_mulr(const cdf &a, float2 w)
{
    const float2 W = bcast(w.x);
    const float2 pn = p2_mul(a.h, bcast(-w.x));
    const float2 e = p2_add(p2_fma(a.h, W, pn), p2_fma(a.h, bcast(w.y), p2_mul(a.l, W)));
    const float2 h = p2_sub(e, pn);                                          // p + e
    return {h, p2_sub(e, p2_add(h, pn))};                                    // e - (h - p)
}
// a + b and a - b, renormalised (df_add on both parts)
__device__ __forceinline__ cdf cdf_add(const cdf &a, const cdf &b)
{
    const float2 s = p2_add(a.h, b.h);
    const float2 bb = p2_sub(s, a.h);
    const float2 e = p2_add(p2_add(p2_add(p2_sub(a.h, p2_sub(s, bb)), p2_sub(b.h, bb)), a.l), b.l);
    const float2 h = p2_add(s, e);
    return {h, p2_sub(e, p2_sub(h, s))};
}
__device__ __forceinline__ cdf cdf_sub(const cdf &a, const cdf &b)
{
    const float2 s = p2_sub(a.h, b.h);
    const float2 bb = p2_sub(s, a.h);                                        // ~ -b.h
    const float2 e = p2_sub(p2_add(p2_sub(p2_sub(a.h, p2_sub(s, bb)), p2_add(b.h, bb)), a.l), b.l);
    const float2 h = p2_add(s, e);
    return {h, p2_sub(e, p2_sub(h, s))};
}

// -v of a complex double by its sign bits (integer operations)
__device__ __forceinline__ double dneg(double x)
{
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}
__device__ __forceinline__ double2 dneg2(double2 v) { return make_double2(dneg(v.x), dneg(v.y)); }


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
// with an element mask (NULL: every pair): only the pairs that touch a masked
// element, and only the tiles that hold one (every warp role applies the same test)
__device__ __forceinline__ bool pair_active(int e, int f, int N, const unsigned char *mask)
{
    return pair_active(e, f, N) && (!mask || mask[e] || mask[f]);
}
// a tile with at least one visited pair
__device__ __forceinline__ bool tile_live(const TileGeo &g, int N) { return g.f0 + 3 >= g.e + 2 && g.f0 < N; }
__device__ __forceinline__ bool tile_live(const TileGeo &g, int N, const unsigned char *mask)
{
    if (!tile_live(g, N)) return false;
    if (!mask || mask[g.e]) return true;
    for (int j = 0; j < 4; ++j)
        if (pair_active(g.e, g.f0 + j, N) && mask[g.f0 + j]) return true;
    return false;
}

template <int N>
__global__ void __launch_bounds__(TC_THREADS, 1)
far_efie_tc_kernel(const __grid_constant__ CUtensorMap bmap, int NE, int Nn, int M, int h, float2 kf,
                   float2 ik2f, float2 sre, float2 sim, const float2 *__restrict__ geo,
                   const unsigned char *__restrict__ emask,
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
                if (!tile_live(tg, NE, emask)) continue;
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
                if (!tile_live(tile_of(t, NE, fgroups), NE, emask)) continue;
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
        // sin^2 of this thread's 8 samples of a stage: 64 aligned bytes (s2f holds Kpad
        // entries), as (hi_j, hi_j+1, lo_j, lo_j+1) for each even j
        const float4 *s2q = reinterpret_cast<const float4 *>(s2f + jq * 8);
        long long gs = 0;
        for (long long t = blockIdx.x; t < ntiles && !*vfailed; t += gridDim.x) {
            const TileGeo tg = tile_of(t, NE, fgroups);
            if (!tile_live(tg, NE, emask)) continue;
            const int f = tg.f0 + ep;
            const bool act = pair_active(tg.e, f, NE, emask);
            TcGreen smp;
            float sc = 0.f;
            if (act) {
                const int p = 4 * tg.e + (pp >> 2), q = 4 * f + (pp & 3);
                const float2 rp = geo[p], zp = geo[P + p], rq = geo[q], zq = geo[P + q];
                const float2 d2 = pair_d2(rp, zp, rq, zq);
                const float2 a2 = df_mul(rp, rq);
                smp.init(d2, make_float2(4.0f * a2.x, 4.0f * a2.y), kf);
                sc = ldexpf(1.0f, bA - row_exp(d2.x));
            }
            const int r_re = ep * 32 + pp, r_im = r_re + 16;
            for (int ks = 0; ks < nst; ++ks, ++gs) {
                const int st = (int)(gs & 1);
                const long long use = gs >> 1;
                if (use > 0 && !mbar_wait(&s.st_empty[st], (uint32_t)((use - 1) & 1))) { fail(); break; }
                if (act) {
                    const int j0 = ks * TK + jq * 8;
                    uint32_t wre[4][ND], wim[4][ND];
                    float4 s4[4];
#pragma unroll
                    for (int i = 0; i < 4; ++i) s4[i] = s2q[ks * (TK / 2) + i];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        // samples j0 + 2i, j0 + 2i + 1; those past h (zero table rows) are zeroed
                        float2 gr, grl, gi, gil;
                        smp.pair(make_float2(s4[i].x, s4[i].y), make_float2(s4[i].z, s4[i].w), s.sc_tab, gr, grl, gi, gil);
                        const float2 live = make_float2(j0 + 2 * i <= h ? 1.0f : 0.0f, j0 + 2 * i + 1 <= h ? 1.0f : 0.0f);
                        split4(p2_mul(gr, live), p2_mul(grl, live), sc, wre[i]);
                        split4(p2_mul(gi, live), p2_mul(gil, live), -sc, wim[i]);
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
        long long ti = 0;
        for (long long t = blockIdx.x; t < ntiles && !*vfailed; t += gridDim.x) {
            const TileGeo tg = tile_of(t, NE, fgroups);
            if (!tile_live(tg, NE, emask)) continue;
            const int e = tg.e, f = tg.f0 + ep;
            const bool act = pair_active(e, f, NE, emask);
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
                    we[lane] = geo[(size_t)(3 + lane / 4) * P + 4 * e + (lane % 4)];
                    wf[lane] = geo[(size_t)(3 + lane / 4) * P + 4 * f + (lane % 4)];
                }
                const int p = 4 * e + (pp >> 2), q = 4 * f + (pp & 3);
                scl = ldexpf(1.0f, row_exp(pair_d2(geo[p], geo[P + p], geo[q], geo[P + q]).x) - bA - sT);
                tre = geo[(size_t)9 * P + 4 * e];
                trf = geo[(size_t)9 * P + 4 * f];
                ttf = df_mul(geo[(size_t)10 * P + 4 * e], geo[(size_t)10 * P + 4 * f]);
            }
            const float2 htt = df_mulf(df_mul(tre, trf), 0.5f), hre = df_mulf(tre, 0.5f), hrf = df_mulf(trf, 0.5f);
            __syncwarp();
            const uint32_t trow = tmem + ((uint32_t)(ep * 32) << 16) + (uint32_t)(set * 4 * N);
            for (int qc = 0; qc < nch; ++qc) {
                const int c_hi = min(CH, nord - qc * CH);      // orders of this chunk
                // (1) orders as double-float words, ACC0 + 2^-8 ACC1 (two-sum, exact) +
                //     2^-16 ACC2 + 2^-24 ACC3, times 2^(e_r - bA - sT)
                if (act) {
                    uint32_t u0[16], u1[16], u2[16], u3[16];
                    tmem_ld16(trow + (uint32_t)(qc * CH), u0);
                    tmem_ld16(trow + (uint32_t)(N + qc * CH), u1);
                    tmem_ld16(trow + (uint32_t)(2 * N + qc * CH), u2);
                    tmem_ld16(trow + (uint32_t)(3 * N + qc * CH), u3);
                    tmem_wait_ld();
                    float a0[16], a1[16], a2[16], a3[16];
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        a0[c] = __uint_as_float(u0[c]);
                        a1[c] = __uint_as_float(u1[c]);
                        a2[c] = __uint_as_float(u2[c]);
                        a3[c] = __uint_as_float(u3[c]);
                    }
#pragma unroll
                    for (int c = 0; c < 16; c += 2) {
                        if (c < c_hi) {
                            const float2 A0 = make_float2(a0[c], a0[c + 1]);
                            const float2 x1 = p2_mul(make_float2(a1[c], a1[c + 1]), bcast(0x1p-8f));
                            const float2 sh = p2_add(A0, x1);
                            const float2 bb = p2_sub(sh, A0);
                            const float2 sl = p2_add(p2_add(p2_sub(A0, p2_sub(sh, bb)), p2_sub(x1, bb)),
                                                     p2_fma(make_float2(a3[c], a3[c + 1]), bcast(0x1p-24f),
                                                            p2_mul(make_float2(a2[c], a2[c + 1]), bcast(0x1p-16f))));
                            const float2 H = p2_mul(sh, bcast(scl)), L = p2_mul(sl, bcast(scl));
                            // (re.hi, im.hi, re.lo, im.lo) of point pair pp: this lane holds part cre
                            float *d0 = reinterpret_cast<float *>(G + ((qc * CH + c) % RING) * SLAB + pp) + cre;
                            d0[0] = H.x;
                            d0[2] = L.x;
                            if (c + 1 < c_hi) {
                                float *d1 = reinterpret_cast<float *>(G + ((qc * CH + c + 1) % RING) * SLAB + pp) + cre;
                                d1[0] = H.y;
                                d1[2] = L.y;
                            }
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
                // (2) contraction: lane = (order, source node b).  The test and the
                //     source vectors of an element are the same six Gauss-point vectors
                //     V = (rho T_a w, T_a w, dRT_a w), so with M = V_e^T G V_f both
                //     orientations read the same 20 entries of M: the forms
                //     (11, dd, ds, sd, ss) of test node a of e and source node b of f
                //     are M's entries ((x, a), (y, b)), and those of the mirror (test
                //     node b of f, source node a of e) are the same entries with ds and
                //     sd exchanged.  Stored once, for orientation 0
                {
                    const int nl = qc * CH + (lane >> 1), b = lane & 1;
                    if ((lane >> 1) < c_hi) {
                        const int slot = nl % RING;
                        const float4 *Gf = G + slot * SLAB;
                        const int o = o0 + nl;
                        const float2 fmf = df_mulf(ik2f, (float)o), fm2f = df_mulf(fmf, (float)o);
                        // G V_f of source node b: (1, s, d) vectors
                        cdf GR1[4], GRs[4], GRd[4];
#pragma unroll
                        for (int g = 0; g < 4; ++g) {
                            cdf r1 = cdf_zero(), rs = r1, rd = r1;
#pragma unroll
                            for (int hq = 0; hq < 4; ++hq) {
                                const cdf gv = cdf_of(Gf[g * 4 + hq]);
                                cdf_mac(r1, gv, wf[(0 + b) * 4 + hq]);
                                cdf_mac(rs, gv, wf[(2 + b) * 4 + hq]);
                                cdf_mac(rd, gv, wf[(4 + b) * 4 + hq]);
                            }
                            GR1[g] = r1;
                            GRs[g] = rs;
                            GRd[g] = rd;
                        }
                        float4 *zl = ZL + slot * ZLS;
#pragma unroll 1
                        for (int a = 0; a < 2; ++a) {
                            cdf acc[5];
#pragma unroll
                            for (int c = 0; c < 5; ++c) acc[c] = cdf_zero();
#pragma unroll
                            for (int g = 0; g < 4; ++g) {
                                const float2 l1 = we[(0 + a) * 4 + g], ls = we[(2 + a) * 4 + g], ld = we[(4 + a) * 4 + g];
                                cdf_mac(acc[0], GR1[g], l1);
                                cdf_mac(acc[1], GRd[g], ld);
                                cdf_mac(acc[2], GRs[g], ld);
                                cdf_mac(acc[3], GRd[g], ls);
                                cdf_mac(acc[4], GRs[g], ls);
                            }
                            // p11, pdd, pds, psd, pss of test node a, source node b -> mode-local parts
                            const int ab = a * 2 + b;
                            P11[slot * P11S + ab] = cdf_f4(acc[0]);
                            zl[0 * 4 + ab] = cdf_f4(cdf_sub(cdf_mulr(acc[0], ttf), cdf_mulr(acc[1], ik2f)));
                            zl[1 * 4 + ab] = cdf_f4(cdf_mj(cdf_mulr(acc[2], fmf)));     // -(j o/k^2) pds
                            zl[2 * 4 + ab] = cdf_f4(cdf_j(cdf_mulr(acc[3], fmf)));      // +(j o/k^2) psd
                            zl[3 * 4 + ab] = cdf_f4(cdf_neg(cdf_mulr(acc[4], fm2f)));
                        }
                    }
                }
                __syncwarp();
                // (3) modes whose orders |m-1|, m, m+1 are all in the ring now: lane =
                //     (mode, a b).  The blocks of orientation 0 (rows e + a, columns
                //     f + b) are tt, t-phi, phi-t, phi-phi = b0..b3; the mirror's
                //     (rows f + b, columns e + a) follow from the exchange of ds and sd
                //     and of the tangents t_rho(e), t_rho(f) in the t-phi / phi-t parts:
                //     b0, -b2, -b1, b3
                const int mlo = (qc == 0) ? m0 : o0 + qc * CH - 1;
                const int mhi = min(m1, o0 + qc * CH + c_hi - 2);
                const int nm = mhi - mlo + 1;
                for (int job = lane; job < 4 * nm; job += 32) {
                    const int ab = job & 3, m = mlo + (job >> 2);
                    const int a = ab >> 1, b = ab & 1;
                    const int sl = (abs(m - 1) - o0) % RING, sm = (m - o0) % RING, sh = (m + 1 - o0) % RING;
                    const cdf lo = cdf_of(P11[sl * P11S + ab]), hi = cdf_of(P11[sh * P11S + ab]);
                    const float4 *zl = ZL + sm * ZLS;
                    const cdf S = cdf_add(lo, hi), D = cdf_sub(lo, hi);
                    cdf bq[4];
                    bq[0] = cdf_add(cdf_mulr(S, htt), cdf_of(zl[0 * 4 + ab]));
                    bq[1] = cdf_add(cdf_mulr(cdf_mj(D), hre), cdf_of(zl[1 * 4 + ab]));
                    bq[2] = cdf_add(cdf_mulr(cdf_j(D), hrf), cdf_of(zl[2 * 4 + ab]));
                    bq[3] = cdf_add(cdf_half(S), cdf_of(zl[3 * 4 + ab]));
                    double2 v[4];
#pragma unroll
                    for (int qb = 0; qb < 4; ++qb) {
                        // (sre + j sim) b
                        const cdf w = cdf_add(cdf_mulr(bq[qb], sre), cdf_mulr(cdf_j(bq[qb]), sim));
                        v[qb] = make_double2(df_to_bits(make_float2(w.h.x, w.l.x)), df_to_bits(make_float2(w.h.y, w.l.y)));
                    }
                    double2 *Zm = Z + (size_t)m * mode_stride;
                    const long long re = e + a, cf = f + b;
#pragma unroll
                    for (int qb = 0; qb < 4; ++qb)
                        catomic_add(Zm + (re + (qb >> 1) * Nn) * ldz + cf + (qb & 1) * Nn, v[qb]);
                    catomic_add(Zm + cf * ldz + re, v[0]);
                    catomic_add(Zm + cf * ldz + re + Nn, dneg2(v[2]));
                    catomic_add(Zm + (cf + Nn) * ldz + re, dneg2(v[1]));
                    catomic_add(Zm + (cf + Nn) * ldz + re + Nn, v[3]);
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
// header: [0] status, [1] sT; then s2f, sin^2 of the Kpad samples as double-float
// words, in pairs of samples (hi_j, hi_j+1, lo_j, lo_j+1); then the digit planes
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
            // sample pairs (j, j + 1), j even, as (hi_j, hi_j+1, lo_j, lo_j+1)
            const double v = (j <= h) ? sin2[j] : 0.0;
            const float hi = (float)v;
            float *w = reinterpret_cast<float *>(s2f) + 4 * (j >> 1) + (j & 1);
            w[0] = hi;
            w[2] = (float)(v - (double)hi);
        }
    }
}

// the geometry rows of the far kernels ([11][P] doubles) as double-float words,
// so that the fill's per-tile set-up runs on the FP32 pipe
constexpr int kGeoRows = 11;
__global__ void tc_geo_kernel(long long n, const double *__restrict__ geo, float2 *__restrict__ gf)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double v = geo[i];
        const float hi = (float)v;
        gf[i] = make_float2(hi, (float)(v - (double)hi));
    }
}

struct TcLayout {
    int N, Npad, Kpad;
    long long s2_off, bd_off, geo_off, bytes;
};

TcLayout tc_layout(int n_elem, int m_max, int nxi)
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
    L.geo_off = ((L.bd_off + 2LL * ND * L.Npad * L.Kpad + 255) / 256) * 256;
    L.bytes = L.geo_off + 8LL * kGeoRows * 4 * n_elem;
    return L;
}

template <int N>
int launch_tc(const TcLayout &L, int NE, int M, int h, float2 kf, float2 ik2f, float2 sre, float2 sim,
              const unsigned char *emask, unsigned char *w, int bA, double2 *Z, long long ldz, long long ms,
              cudaStream_t st)
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
    kern<<<grid, TC_THREADS, smem, st>>>(map, NE, NE + 1, M, h, kf, ik2f, sre, sim,
                                         reinterpret_cast<const float2 *>(w + L.geo_off), emask,
                                         reinterpret_cast<const float2 *>(w + L.s2_off),
                                         reinterpret_cast<const int *>(w), bA, Z, ldz, ms,
                                         reinterpret_cast<int *>(w));
    return check_launch("far_efie_tc");
}

}  // namespace
}  // namespace gb

extern "C" long long ghost_bor_far_efie_tc_workspace(int n_elem, int m_max, int nxi)
{
    if (n_elem < 0 || m_max < 0 || nxi < 2 || (nxi & 1)) return -1;
    return gb::tc_layout(n_elem, m_max, nxi).bytes;
}

extern "C" int ghost_bor_far_efie_tc_tables(int m_max, int nxi, const double *dct, const double *sin2,
                                            void *work, long long work_bytes, void *stream)
{
    using namespace gb;
    if (m_max < 0 || nxi < 2 || (nxi & 1) || !dct || !sin2 || !work ||
        (reinterpret_cast<uintptr_t>(work) & 255) || work_bytes < ghost_bor_far_efie_tc_workspace(0, m_max, nxi))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const TcLayout L = tc_layout(0, m_max, nxi);
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

extern "C" int ghost_bor_far_efie_tc_masked(int n_elem, int m_max, int nxi, double k, double scale_re,
                                            double scale_im, const double *geo, const unsigned char *elem_mask,
                                            void *work, long long work_bytes, void *Z, long long ldz,
                                            long long mode_stride, void *stream)
{
    using namespace gb;
    if (n_elem < 3 || m_max < 0 || nxi < 2 || (nxi & 1) || !geo || !Z || !work ||
        (reinterpret_cast<uintptr_t>(work) & 255) || work_bytes < ghost_bor_far_efie_tc_workspace(n_elem, m_max, nxi) ||
        ldz < 2LL * (n_elem + 1) || mode_stride < ldz * 2LL * (n_elem + 1) || !(k > 0.0))
        return GHOST_BOR_EINVAL;
    const int h = nxi / 2;
    // level-0 products d0 t0 (|d0| <= 2^bA, |t0| <= 128) summed over h + 1 samples stay below 2^24
    int bA = 7;
    while (bA > 1 && (long long)(h + 1) << (bA + 7) > (1LL << 24)) --bA;
    if ((long long)(h + 1) << (bA + 7) > (1LL << 24)) return GHOST_BOR_EUNSUPPORTED;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const TcLayout L = tc_layout(n_elem, m_max, nxi);
    unsigned char *w = reinterpret_cast<unsigned char *>(work);
    const long long ng = (long long)kGeoRows * 4 * n_elem;
    tc_geo_kernel<<<(int)((ng + 255) / 256 < 1024 ? (ng + 255) / 256 : 1024), 256, 0, st>>>(
        ng, geo, reinterpret_cast<float2 *>(w + L.geo_off));
    const int rc = check_launch("far_efie_tc: geometry words");
    if (rc) return rc;
    auto split = [](double v) {
        const float hi = (float)v;
        return make_float2(hi, (float)(v - (double)hi));
    };
    const float2 kf = split(k), ik2f = split(1.0 / (k * k)), sre = split(scale_re), sim = split(scale_im);
    double2 *Zd = reinterpret_cast<double2 *>(Z);
    if (L.N == 32) return launch_tc<32>(L, n_elem, m_max, h, kf, ik2f, sre, sim, elem_mask, w, bA, Zd, ldz, mode_stride, st);
    if (L.N == 64) return launch_tc<64>(L, n_elem, m_max, h, kf, ik2f, sre, sim, elem_mask, w, bA, Zd, ldz, mode_stride, st);
    return launch_tc<128>(L, n_elem, m_max, h, kf, ik2f, sre, sim, elem_mask, w, bA, Zd, ldz, mode_stride, st);
}

extern "C" int ghost_bor_far_efie_tc(int n_elem, int m_max, int nxi, double k, double scale_re, double scale_im,
                                     const double *geo, void *work, long long work_bytes,
                                     void *Z, long long ldz, long long mode_stride, void *stream)
{
    return ghost_bor_far_efie_tc_masked(n_elem, m_max, nxi, k, scale_re, scale_im, geo, nullptr, work, work_bytes,
                                        Z, ldz, mode_stride, stream);
}
