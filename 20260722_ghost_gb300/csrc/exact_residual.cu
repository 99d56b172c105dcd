// exact_residual.cu -- refinement residual R = B - (Z_far + Z_near) X with
// exact products on the bf16 tensor cores (Ozaki splitting).
//
// Z_far (complex double) is viewed as the real matrix A [n][2n] (re, im
// interleaved) and X (the FP32 solution) through the 2x2 real expansion
// Bt[2j+r][2k+c] = [[Xr, -Xi], [Xi, Xr]][r][c] (as in tc_gemm.cu), so that
// A Bt^T is the interleaved storage of Z_far X.
//
// Splitting: every row i of A gets a power-of-two scale 2^e_i >= its largest
// magnitude, every complex column j of X a scale 2^f_j; each scaled value u
// (|u| < 1) is written as q1 2^-7 + q2 2^-15 + q3 2^-23 + q4 2^-31 (+ q5 2^-39
// for A) with integers |q_s| <= 128 (balanced base-256 digits), which bf16
// holds exactly.  A takes five digits: most entries of a row are far below
// its largest (the near-diagonal blocks), and with four the truncation,
// 2^-32 of the row scale, left ~2.6e-8 of ||B|| in the residual of the
// 1200-segment cone-sphere -- the floor of the refined far field; four digits
// hold the FP32 solution's entries within 2^-8 of their column scale exactly.
// A product q_s q_t (|.| <= 2^14) is exact in the FP32 accumulator, and so is
// any sum of them below 2^24: the slice pairs with the same s + t share one
// TMEM accumulator ("level" L = s + t - 2, scale 2^(-14 - 8 L)), at most four
// pairs per level, accumulated over K chunks of 192 real columns
// (192 * 4 * 2^14 < 2^24).  After each chunk the five levels are folded into
// double-float (hi, lo) register accumulators; pairs with s + t > 6 are
// dropped (below 2^-40 of the row and column scales).  The result carries
// ~2^-40 of the row scales and ~2^-32 of the column scales -- far below the
// FP32-product floor (~2^-24) of a split-word SIMT residual -- and runs at
// tensor-core rate.
//
// The near band is added to Z_far before the split (A = Z_far + band), so the
// epilogue only forms R = B - P in FP64 and zeroes the masked rows.
//
// Kernel (one CTA per 128 rows x 48 complex right-hand sides): warp 0 streams
// the A and Bt slices of each 32-deep K stage through a three-stage ring (TMA,
// 64-byte swizzle); warp 1 issues the 14 slice-pair MMAs (M = 128, N = 96) per
// 16 K into the five level accumulators (5 x 96 TMEM columns); warps 2..13 fold
// each finished K chunk into the double-float accumulators and release TMEM as
// soon as the chunk is in registers.  The wide N halves the shared-memory
// reads of the A slices per output column, which bound the MMA issue rate at
// N = 48.  All waits are bounded.
#include <cuda_bf16.h>

#include "common.cuh"
#include "tcgen05.cuh"

namespace gb {
namespace {

constexpr int XSA = 5;                   // slices of A (Z_far rows)
constexpr int XS = 4;                    // slices of Bt (the FP32 solution: 4 slices hold it exactly)
constexpr int XBM = 128;                 // tile rows
constexpr int XBN = 96;                  // tile real columns (48 complex rhs)
constexpr int XBK = 32;                  // real K per stage (32 bf16 = one 64-byte swizzle row)
constexpr int XSTAGES = 3;               // operand ring depth
constexpr int XCHUNK = 6;                // stages per exact accumulation (K = 192)
constexpr int XLEV = 5;                  // levels s + t = 2..6
constexpr uint32_t XTMEM_COLS = 512;     // one accumulator set of 5 x 96 columns
// warps: 0 TMA, 1 MMA, 2..13 fold.  A fold warp reads the TMEM lanes of its rank
// in its warpgroup, 32 (warp % 4) .. + 31, and one of three 32-column groups
// (14 warps: at most 4 per SM sub-partition, 128 registers each)
constexpr int XW_FOLD0 = 2, XNFOLD = 12;
constexpr int XTHREADS = (XW_FOLD0 + XNFOLD) * 32;
constexpr int XCOLS = XBN / 3;           // real columns per fold thread
// the slice pairs (A slice, Bt slice) with s + t = 2..6, level by level, and
// whether a pair is the first of its level (its first MMA of a chunk overwrites)
constexpr int XPAIRS = 14;
__device__ constexpr int kPairA[XPAIRS] = {1, 1, 2, 1, 2, 3, 1, 2, 3, 4, 2, 3, 4, 5};
__device__ constexpr int kPairB[XPAIRS] = {1, 2, 1, 3, 2, 1, 4, 3, 2, 1, 4, 3, 2, 1};
__device__ constexpr bool kPairFirst[XPAIRS] = {true, true, false, true, false, false, true, false, false, false,
                                                true, false, false, false};
constexpr int XA_TILE = XBM * XBK;       // bf16 elements
constexpr int XB_TILE = XBN * XBK;

struct __align__(1024) XSmem {
    __nv_bfloat16 a[XSTAGES][XSA][XA_TILE];    // 3 stages x 5 slices x 8 KB
    __nv_bfloat16 b[XSTAGES][XS][XB_TILE];     // 3 stages x 4 slices x 6 KB
    unsigned long long full[XSTAGES], empty[XSTAGES], tfull, tempty, drain;
    uint32_t tmem_base;
    int failed;
};
static_assert(sizeof(XSmem) + 1024 <= 227 * 1024, "exact residual shared memory");
static_assert(XBM * (XBN + 1) * sizeof(double) <= sizeof(__nv_bfloat16) * XSTAGES * XSA * XA_TILE,
              "the P tile fits in the A stages");

// instruction descriptor: D f32, A/B bf16 (kind::f16), both K-major, M = 128, N = 64
constexpr uint32_t kIdescBf16 = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(XBN >> 3) << 17) |
                                ((uint32_t)(XBM >> 4) << 24);

// UMMA shared-memory descriptor: K-major operand, 64-byte swizzle, 8-row
// groups 512 bytes apart (SBO), version 1
__device__ __forceinline__ uint64_t umma_desc_sw64x(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)((512u >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)4u << 61;             // SWIZZLE_64B
    return d;
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                 ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kIdescBf16), "r"(accumulate));
}

// exponent e with |v| < 2^e for every |v| <= m (m > 0); 0 for m = 0
__device__ __forceinline__ int scale_exp(double m)
{
    if (!(m > 0.0)) return 0;
    int e;
    frexp(m, &e);                        // m = f 2^e, f in [0.5, 1)
    return e;
}

// four balanced base-256 digits of v / 2^e (|v| < 2^e):
//   v / 2^e ~ q1 2^-7 + q2 2^-15 + q3 2^-23 + q4 2^-31,  |q_s| <= 128,
// by integer arithmetic on the IEEE bits: W = round(v 2^(31 - e)) (|W| <= 2^31)
// is split into balanced base-256 digits with arithmetic shifts.
template <int NS>
__device__ __forceinline__ void digits(double v, int e, float (&q)[NS])
{
    const long long bits = __double_as_longlong(v);
    const int E = (int)((bits >> 52) & 0x7ff);
    long long W = 0;
    if (E != 0) {                                    // zero and subnormals -> 0 (below 2^-1022)
        const long long m = (bits & 0xfffffffffffffLL) | 0x10000000000000LL;
        const int sh = (E - 1075) + (8 * NS - 1) - e;  // v = m 2^(E - 1075)
        if (sh >= 0) W = m << sh;
        else if (sh > -64) W = (m + (1LL << (-sh - 1))) >> (-sh);
        if (bits < 0) W = -W;
    }
#pragma unroll
    for (int s = NS - 1; s >= 1; --s) {
        const long long t = (W + 128) >> 8;          // floor((W + 128) / 256)
        q[s] = (float)(int)(W - (t << 8));
        W = t;
    }
    q[0] = (float)(int)W;
}

// the same for an FP32 value (exact FP32 arithmetic)
__device__ __forceinline__ void digits(float v, int e, float (&q)[XS])
{
    float t = ldexpf(v, 7 - e);
#pragma unroll
    for (int s = 0; s < XS; ++s) {
        const float d = rintf(t);
        q[s] = d;
        t = (t - d) * 256.0f;
    }
}

// near band entry of A = Z_far + band at (row i, complex column k), or 0
__device__ __forceinline__ double2 band_at(const double2 *band, int b, int Nn, int i, int k)
{
    if (!band) return make_double2(0.0, 0.0);
    const int half = i >= Nn ? 1 : 0, node = i - half * Nn;
    const int ch = k >= Nn ? 1 : 0, jn = k - ch * Nn;
    const int d = jn - node + 2;
    if (d < 0 || d > 4) return make_double2(0.0, 0.0);
    return band[(((size_t)b * 4 + 2 * half + ch) * Nn + node) * 5 + d];
}

// row exponents of A: one warp per row of Z_far (2n reals)
__global__ void row_exp_kernel(int batch, int n, int Nn, const double2 *__restrict__ Z, long long ldz, long long sz,
                               const double2 *__restrict__ band, int *__restrict__ ex)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= batch * n) return;
    const int b = warp / n, i = warp % n;
    const double2 *row = Z + (size_t)b * sz + (size_t)i * ldz;
    double m = 0.0;
    for (int k = lane; k < n; k += 32) {
        const double2 v = cadd(row[k], band_at(band, b, Nn, i, k));
        m = fmax(m, fmax(fabs(v.x), fabs(v.y)));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    if (lane == 0) ex[warp] = scale_exp(m);
}

// A slices: As[s][b][i][kr], kr < Kp (zero beyond 2n)
__global__ void slice_a_kernel(int batch, int n, int Nn, int Kp, const double2 *__restrict__ Z, long long ldz,
                               long long sz, const double2 *__restrict__ band, const int *__restrict__ ex,
                               __nv_bfloat16 *__restrict__ As)
{
    const int kh = Kp / 2;
    const long long total = (long long)batch * n * kh;
    const size_t plane = (size_t)batch * n * Kp;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(idx % kh);
        const long long bi = idx / kh;
        const int i = (int)(bi % n), b = (int)(bi / n);
        const double2 v = (k < n) ? cadd(Z[(size_t)b * sz + (size_t)i * ldz + k], band_at(band, b, Nn, i, k))
                                  : make_double2(0.0, 0.0);
        const int e = ex[bi];
        float qr[XSA], qi[XSA];
        digits(v.x, e, qr);
        digits(v.y, e, qi);
        const size_t o = (size_t)bi * Kp + 2 * (size_t)k;
#pragma unroll
        for (int s = 0; s < XSA; ++s) {
            __nv_bfloat162 w;
            w.x = __float2bfloat16_rn(qr[s]);
            w.y = __float2bfloat16_rn(qi[s]);
            *reinterpret_cast<__nv_bfloat162 *>(As + s * plane + o) = w;
        }
    }
}

// column exponents of X (FP32 solution [b][k][j], k < n, j < nrhs)
__global__ void col_exp_kernel(int n, int nrhs, const float2 *__restrict__ X, long long ldx, long long sx,
                               int *__restrict__ fx)
{
    __shared__ float red[8][33];
    const int j = blockIdx.x * 32 + (threadIdx.x & 31), ty = threadIdx.x >> 5, b = blockIdx.y;
    float m = 0.f;
    if (j < nrhs)
        for (int k = ty; k < n; k += 8) {
            const float2 v = X[(size_t)b * sx + (size_t)k * ldx + j];
            m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
        }
    red[ty][threadIdx.x & 31] = m;
    __syncthreads();
    if (ty == 0 && j < nrhs) {
        for (int r = 1; r < 8; ++r) m = fmaxf(m, red[r][threadIdx.x]);
        fx[(size_t)b * nrhs + j] = scale_exp((double)m);
    }
}

// Bt slices: Bs[s][b][2j + r][kr] with Bt[2j+r][2k+c] = [[Xr, -Xi], [Xi, Xr]][r][c];
// 32 x 32 complex tiles transposed through shared memory
__global__ void __launch_bounds__(256)
slice_b_kernel(int batch, int n, int nrhs, int Kp, const float2 *__restrict__ X, long long ldx, long long sx,
               const int *__restrict__ fx, __nv_bfloat16 *__restrict__ Bs)
{
    __shared__ float2 t[32][33];
    const int j0 = blockIdx.x * 32, k0 = blockIdx.y * 32, b = blockIdx.z;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r = ty; r < 32; r += 8) {
        const int k = k0 + r, j = j0 + tx;
        t[r][tx] = (k < n && j < nrhs) ? X[(size_t)b * sx + (size_t)k * ldx + j] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const size_t plane = (size_t)batch * 2 * nrhs * Kp;
    for (int q = threadIdx.x; q < 64 * 64; q += 256) {
        const int orow = q / 64, ocol = q % 64;
        const int j = j0 + orow / 2, rr = orow & 1;
        const int kc = k0 * 2 + ocol;
        if (j >= nrhs || kc >= Kp) continue;
        const float2 x = t[ocol / 2][orow / 2];
        const int c = ocol & 1;
        const float v = (rr == 0) ? (c == 0 ? x.x : -x.y) : (c == 0 ? x.y : x.x);
        float qd[XS];
        digits(v, fx[(size_t)b * nrhs + j], qd);
        const size_t o = ((size_t)b * 2 * nrhs + 2 * j + rr) * Kp + kc;
#pragma unroll
        for (int s = 0; s < XS; ++s) Bs[s * plane + o] = __float2bfloat16_rn(qd[s]);
    }
}

// 2^k as a double (|k| < 1023), built from the exponent bits
__device__ __forceinline__ double exp2i(int k)
{
    return __longlong_as_double((long long)(k + 1023) << 52);
}

__device__ __forceinline__ bool row_masked(const int *mr, int r)
{
    return mr[0] == r || mr[1] == r || mr[2] == r || mr[3] == r;
}

struct XMaps {
    CUtensorMap a[XSA];
    CUtensorMap b[XS];
};

__global__ void __launch_bounds__(XTHREADS, 1)
exact_residual_kernel(const __grid_constant__ XMaps maps, int n, int nrhs, int Kp,
                      const int *__restrict__ ex, const int *__restrict__ fx, const int *__restrict__ mask_rows,
                      const double2 *__restrict__ B, long long ldb, long long sbb,
                      double2 *__restrict__ R, float2 *__restrict__ R32, double *__restrict__ norms,
                      int *__restrict__ err)
{
    extern __shared__ unsigned char smem_raw[];
    XSmem &s = *reinterpret_cast<XSmem *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n0 = blockIdx.x * XBN, m0 = blockIdx.y * XBM, b = blockIdx.z;
    const int nst = Kp / XBK;
    const int nch = (nst + XCHUNK - 1) / XCHUNK;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&s.tmem_base)), "r"(XTMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < XSTAGES; ++i) {
            mbar_init(&s.full[i], 1);
            mbar_init(&s.empty[i], 1);
        }
        mbar_init(&s.tfull, 1);
        mbar_init(&s.tempty, XNFOLD);
        mbar_init(&s.drain, 1);
        s.failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s.tmem_base;
    volatile int *vfailed = &s.failed;
    auto fail = [&]() {
        *vfailed = 1;
        atomicExch(err, 1);
    };

    if (warp == 0) {
        // ---------------- TMA: the A and Bt slices of each 32-deep K stage into a 3-stage ring
        if (lane == 0) {
            const uint32_t stage_bytes = (uint32_t)((XSA * XA_TILE + XS * XB_TILE) * 2);
            int ks = 0;
            for (; ks < nst && !*vfailed; ++ks) {
                const int st = ks % XSTAGES;
                const int use = ks / XSTAGES;
                if (use > 0 && !mbar_wait(&s.empty[st], (uint32_t)((use - 1) & 1))) { fail(); break; }
                mbar_expect_tx(&s.full[st], stage_bytes);
#pragma unroll
                for (int q = 0; q < XSA; ++q) tma_load_3d(s.a[st][q], &maps.a[q], ks * XBK, m0, b, &s.full[st]);
#pragma unroll
                for (int q = 0; q < XS; ++q) tma_load_3d(s.b[st][q], &maps.b[q], ks * XBK, n0, b, &s.full[st]);
            }
            // drain: every issued copy has landed before the CTA may exit
            for (int st = 0; st < XSTAGES; ++st) {
                const int n_issued = ks > st ? (ks - st + XSTAGES - 1) / XSTAGES : 0;
                if (n_issued > 0 && !mbar_wait(&s.full[st], (uint32_t)((n_issued - 1) & 1))) fail();
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA: the K chunks into the accumulator set, one chunk at a time
        if (lane == 0) {
            int ks = 0;
            bool ok = true;
            // stage-0 descriptors; stage st lies st times a fixed number of 16-byte units further
            uint64_t adesc[XSA], bdesc[XS];
#pragma unroll
            for (int q = 0; q < XSA; ++q) adesc[q] = umma_desc_sw64x(smem_u32(s.a[0][q]));
#pragma unroll
            for (int q = 0; q < XS; ++q) bdesc[q] = umma_desc_sw64x(smem_u32(s.b[0][q]));
            constexpr uint32_t kAStage = XSA * XA_TILE * 2 / 16, kBStage = XS * XB_TILE * 2 / 16;
            for (int c = 0; c < nch && ok && !*vfailed; ++c) {
                // the fold has read the previous chunk's accumulators
                if (c >= 1 && !mbar_wait(&s.tempty, (uint32_t)((c - 1) & 1))) { ok = false; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const int k_lo = c * XCHUNK, k_hi = min(nst, k_lo + XCHUNK);
                for (; ks < k_hi; ++ks) {
                    const int st = ks % XSTAGES;
                    if (!mbar_wait(&s.full[st], (uint32_t)((ks / XSTAGES) & 1))) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const bool first = ks == k_lo;
                    const uint32_t aoff = (uint32_t)st * kAStage, boff = (uint32_t)st * kBStage;
                    // 14 slice pairs by level; the descriptors step by 32 bytes (2 units)
                    // per 16-deep MMA
#pragma unroll
                    for (int pr = 0; pr < XPAIRS; ++pr) {
                        const int sa = kPairA[pr], sb = kPairB[pr], L = sa + sb - 2;
                        const uint64_t ad = adesc[sa - 1] + aoff, bd = bdesc[sb - 1] + boff;
#pragma unroll
                        for (int kk = 0; kk < XBK / 16; ++kk) {
                            const uint32_t acc = (!first || !kPairFirst[pr] || kk > 0) ? 1u : 0u;
                            umma_bf16(tmem + (uint32_t)(L * XBN), ad + 2u * kk, bd + 2u * kk, acc);
                        }
                    }
                    umma_commit(&s.empty[st]);          // the stage may be refilled once these MMAs are done
                }
                if (!ok) break;
                umma_commit(&s.tfull);                  // the chunk's accumulators are complete
            }
            if (!ok) fail();
            // drain: every issued MMA has completed before TMEM is freed
            umma_commit(&s.drain);
            if (!mbar_wait(&s.drain, 0)) fail();
        }
    }

    // ---------------- fold: each chunk's five exact levels into double-float
    // (hi, lo) accumulators of this thread's row (TMEM lane 32 (warp % 4) + lane)
    // and 32 of the tile's 96 real columns; the TMA warp keeps loading the next
    // chunk's stages meanwhile, and the MMAs of the next chunk start as soon as
    // the last level is in registers
    const int fw = warp - XW_FOLD0;
    const int quad = warp & 3, cg = fw >> 2;        // fold warps 2..13: every (quad, cg) once
    float hi[XCOLS], lo[XCOLS];
#pragma unroll
    for (int c = 0; c < XCOLS; ++c) { hi[c] = 0.f; lo[c] = 0.f; }
    if (warp >= XW_FOLD0) {
        for (int c = 0; c < nch && !*vfailed; ++c) {
            if (!mbar_wait(&s.tfull, (uint32_t)(c & 1))) { fail(); break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t row_addr = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(cg * XCOLS);
#pragma unroll
            for (int L = 0; L < XLEV; ++L) {
                float v[32];
                tmem_ld32(row_addr + (uint32_t)(L * XBN), v);
                if (L == XLEV - 1) {
                    // every level of this chunk is read: the set may take the next chunk
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&s.tempty);
                }
                const float sc = ldexpf(1.0f, -14 - 8 * L);
#pragma unroll
                for (int q = 0; q < XCOLS; ++q) {
                    // x is exact (an integer times a power of two); a two-sum keeps
                    // every level exact in (hi, lo), so lo only collects rounding
                    // errors of hi (~2^-24 |hi|) and stays precise
                    const float x = v[q] * sc;
                    const float t = hi[q] + x;
                    const float bb2 = t - hi[q];
                    lo[q] += (hi[q] - (t - bb2)) + (x - bb2);
                    hi[q] = t;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();                             // every copy, MMA and fold is done: the stages are free
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // P = 2^(e_i + f_j) (hi + lo) through shared memory (the operand buffers are free)
    double (*Ps)[XBN + 1] = reinterpret_cast<double (*)[XBN + 1]>(&s.a[0][0][0]);
    const bool good = !*vfailed;
    if (good && warp >= XW_FOLD0) {
        const int r = quad * 32 + lane;
        const int i = m0 + r;
        const int e = (i < n) ? ex[(size_t)b * n + i] : 0;
#pragma unroll
        for (int c = 0; c < XCOLS; ++c) {
            const int cc = cg * XCOLS + c;
            const int j = (n0 + cc) >> 1;
            const int f = (j < nrhs) ? fx[(size_t)b * nrhs + j] : 0;
            Ps[r][cc] = ((double)hi[c] + (double)lo[c]) * exp2i(e + f);
        }
    }
    __syncthreads();
    // R = B - P (the near band is inside the slices), masked rows zero; fold warp
    // fw takes rows fw, fw + 12, ..., lane = complex column (48 per tile, two
    // passes); norms in FP32 (reported, not refined)
    float rn = 0.f, bn = 0.f;
    if (good && warp >= XW_FOLD0) {
        const int *mr = mask_rows + 4 * b;
        const double2 *Bb = B + (size_t)b * sbb;
        for (int jc = lane; jc < XBN / 2; jc += 32) {
            const int j = (n0 >> 1) + jc;
            for (int r = fw; r < XBM; r += XNFOLD) {
                const int i = m0 + r;
                if (i >= n || j >= nrhs) continue;
                const double2 bv = Bb[(size_t)i * ldb + j];
                double2 rv = make_double2(bv.x - Ps[r][2 * jc], bv.y - Ps[r][2 * jc + 1]);
                if (row_masked(mr, i)) rv = make_double2(0.0, 0.0);
                if (R) R[(size_t)b * sbb + (size_t)i * ldb + j] = rv;
                const float2 r32 = make_float2((float)rv.x, (float)rv.y);
                if (R32) R32[(size_t)b * sbb + (size_t)i * ldb + j] = r32;
                const float2 b32 = make_float2((float)bv.x, (float)bv.y);
                rn = fmaf(r32.x, r32.x, fmaf(r32.y, r32.y, rn));
                bn = fmaf(b32.x, b32.x, fmaf(b32.y, b32.y, bn));
            }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        rn += __shfl_xor_sync(0xffffffffu, rn, off);
        bn += __shfl_xor_sync(0xffffffffu, bn, off);
    }
    if (lane == 0 && good && warp >= XW_FOLD0) {
        atomicAdd(norms + 2 * b, (double)rn);
        atomicAdd(norms + 2 * b + 1, (double)bn);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(XTMEM_COLS));
    }
}

// K-major [batch][rows][Kp] bf16 operand, box 32 x box_rows, 64-byte swizzle
bool make_map_bf16(CUtensorMap *map, const __nv_bfloat16 *base, int rows, int Kp, int batch, int box_rows)
{
    auto enc = get_encode();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)batch};
    const cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)rows * Kp * 2};
    const cuuint32_t box[3] = {XBK, (cuuint32_t)box_rows, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16 *>(base), dims, strides, box,
               estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

long long kp_of(int n) { return ((2LL * n + XBK - 1) / XBK) * XBK; }

}  // namespace
}  // namespace gb

// Workspace: [0, 256) status int (1 = a bounded wait gave up), then row and
// column exponents, then the A and Bt slices (256-byte aligned blocks).
extern "C" long long ghost_bor_residual_exact_workspace(int batch, int n, int nrhs)
{
    if (batch < 1 || n < 1 || nrhs < 1) return -1;
    using namespace gb;
    const long long Kp = kp_of(n);
    auto up = [](long long x) { return (x + 255) / 256 * 256; };
    return 256 + up(4LL * batch * n) + up(4LL * batch * nrhs) + up(2LL * XSA * batch * n * Kp) +
           up(2LL * XS * batch * 2 * nrhs * Kp);
}

extern "C" int ghost_bor_residual_exact(int batch, int n, int nrhs, int Nn,
                                        const double *Zf, long long ldz, long long stride_z,
                                        const double *band, const int *mask_rows,
                                        const float *X32, const double *B, long long ldb, long long stride_b,
                                        double *R, float *R32, double *norms,
                                        void *work, long long work_bytes, void *stream)
{
    using namespace gb;
    if (batch < 1 || n < 1 || nrhs < 1 || !Zf || !mask_rows || !X32 || !B || (!R && !R32) || !norms ||
        ldz < n || ldb < nrhs || n != 2 * Nn || !work || (reinterpret_cast<uintptr_t>(work) & 255) ||
        work_bytes < ghost_bor_residual_exact_workspace(batch, n, nrhs))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int Kp = (int)kp_of(n);
    auto up = [](long long x) { return (x + 255) / 256 * 256; };
    unsigned char *w = reinterpret_cast<unsigned char *>(work);
    int *errp = reinterpret_cast<int *>(w);
    int *ex = reinterpret_cast<int *>(w + 256);
    int *fx = reinterpret_cast<int *>(w + 256 + up(4LL * batch * n));
    __nv_bfloat16 *As = reinterpret_cast<__nv_bfloat16 *>(w + 256 + up(4LL * batch * n) + up(4LL * batch * nrhs));
    __nv_bfloat16 *Bs = As + up(2LL * XSA * batch * n * Kp) / 2;
    const size_t aplane = (size_t)batch * n * Kp, bplane = (size_t)batch * 2 * nrhs * Kp;

    if (cudaMemsetAsync(errp, 0, sizeof(int), st) != cudaSuccess ||
        cudaMemsetAsync(norms, 0, sizeof(double) * 2 * batch, st) != cudaSuccess)
        return check_launch("residual_exact: memset");
    const double2 *Z = reinterpret_cast<const double2 *>(Zf);
    const float2 *X = reinterpret_cast<const float2 *>(X32);
    {
        const long long rows = (long long)batch * n;
        const double2 *bd = reinterpret_cast<const double2 *>(band);
        row_exp_kernel<<<(unsigned)((rows * 32 + 255) / 256), 256, 0, st>>>(batch, n, Nn, Z, ldz, stride_z, bd, ex);
        int rc = check_launch("residual_exact: row exponents");
        if (rc) return rc;
        const long long pairs = (long long)batch * n * (Kp / 2);
        const int blocks = (int)((pairs + 255) / 256 < 152 * 32 ? (pairs + 255) / 256 : 152 * 32);
        slice_a_kernel<<<blocks, 256, 0, st>>>(batch, n, Nn, Kp, Z, ldz, stride_z, bd, ex, As);
        if ((rc = check_launch("residual_exact: slice A"))) return rc;
        dim3 gc((nrhs + 31) / 32, batch);
        col_exp_kernel<<<gc, 256, 0, st>>>(n, nrhs, X, ldb, stride_b, fx);
        if ((rc = check_launch("residual_exact: column exponents"))) return rc;
        dim3 gb2((nrhs + 31) / 32, (Kp / 2 + 31) / 32, batch);
        slice_b_kernel<<<gb2, 256, 0, st>>>(batch, n, nrhs, Kp, X, ldb, stride_b, fx, Bs);
        if ((rc = check_launch("residual_exact: slice B"))) return rc;
    }
    XMaps maps;
    for (int q = 0; q < XSA; ++q) {
        if (!make_map_bf16(&maps.a[q], As + q * aplane, n, Kp, batch, XBM) ||
            (q < XS && !make_map_bf16(&maps.b[q], Bs + q * bplane, 2 * nrhs, Kp, batch, XBN))) {
            set_last_error("residual_exact: cuTensorMapEncodeTiled failed");
            return GHOST_BOR_ECUDA;
        }
    }
    const size_t smem = sizeof(XSmem) + 1024;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(exact_residual_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return check_launch("residual_exact: smem attribute");
        attr = true;
    }
    dim3 grid((2 * nrhs + XBN - 1) / XBN, (n + XBM - 1) / XBM, batch);
    exact_residual_kernel<<<grid, XTHREADS, smem, st>>>(maps, n, nrhs, Kp, ex, fx, mask_rows,
                                                         reinterpret_cast<const double2 *>(B), ldb, stride_b,
                                                         reinterpret_cast<double2 *>(R),
                                                         reinterpret_cast<float2 *>(R32), norms, errp);
    return check_launch("residual_exact");
}
