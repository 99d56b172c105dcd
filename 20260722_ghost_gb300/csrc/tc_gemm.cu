// tc_gemm.cu -- complex FP32 GEMM update C -= A B on the 5th-generation tensor
// cores (tcgen05, kind::tf32, accumulator in TMEM, operands staged by TMA).
//
// Used for the trailing updates of the batched LU and the block updates of the
// triangular solves (bor_solver.py:753 replaced by ghost_bor_getrf/getrs).
//
// Precision: 3xTF32.  Each FP32 operand x is split into hi = tf32(x) and
// lo = x - hi; the product is hi*hi + hi*lo + lo*hi accumulated in FP32 (the
// lo*lo term is below FP32 rounding).  This keeps the LU accurate to FP32
// level, which the FP64 refinement of the solution needs.
//
// Complex arithmetic as one real GEMM: the FP32 storage of a complex row-major
// matrix A [M][K] is the real matrix A_r [M][2K] (re, im interleaved).  With
// B expanded into 2x2 real blocks B''[2k+c][2n+r] = [[Br, Bi], [-Bi, Br]][c][r]
// the real product A_r B'' is the interleaved storage of A B.  The GEMM runs
// D[M][2N] = A_r [M][2K] x Bt [2N][2K]^T with both operands K-major.
//
// Tiles: 128 x 128 output (M x 2N real), K in stages of 32 (one 128-byte
// swizzle row), 3 stages.  The kernel is persistent (one CTA per SM walks the
// tiles) and warp-specialised: warp 0 issues the TMA loads, warp 1 the MMAs
// into one of two TMEM accumulators, and warps 2..5 drain the other
// accumulator (tcgen05.ld, C -= acc), so the epilogue of one tile overlaps
// the main loop of the next.
#include "common.cuh"
#include "tcgen05.cuh"

namespace gb {
namespace {

constexpr int BM = 128, BNR = 128, BK = 32;       // tile rows, tile real columns, K per stage
constexpr int STAGES = 3;
constexpr int TILE_FLOATS = BM * BK;               // 16 KB per operand tile
constexpr int TC_THREADS = 192;                    // producer, MMA, 4 epilogue warps
constexpr uint32_t TMEM_COLS = 256;                // two 128-column accumulators

// polls of each pipeline mbarrier wait before the kernel gives up (the drains
// of copies and MMAs in flight keep WAIT_LIMIT); set by ghost_bor_set_wait_limit
long long g_pipeline_wait_limit = WAIT_LIMIT;

struct __align__(1024) TcSmem {
    float a_hi[STAGES][TILE_FLOATS];
    float a_lo[STAGES][TILE_FLOATS];
    float b_hi[STAGES][TILE_FLOATS];
    float b_lo[STAGES][TILE_FLOATS];
    // epilogue staging, 8 KB per epilogue warp: two 32 x 32 FP32 boxes of -acc
    // in the 128-byte swizzled layout of the C tensor map (TMA reduce-add
    // path), or one 32 x 33 transpose (load/store path)
    float ep[4][2][32 * 32];
    unsigned long long full[STAGES];               // TMA -> MMA
    unsigned long long empty[STAGES];              // MMA -> TMA (tcgen05.commit)
    unsigned long long tfull[2];                   // MMA -> epilogue (tcgen05.commit)
    unsigned long long tempty[2];                  // epilogue -> MMA (4 warp arrivals)
    unsigned long long drain;                      // MMA drain on the error path
    uint32_t tmem_base;
    int failed;
};

// instruction descriptor: D f32, A/B tf32, both K-major, M = 128, N = 128
constexpr uint32_t kIdescTf32 = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BNR >> 3) << 17) |
                                ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n"
                 ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kIdescTf32), "r"(accumulate));
}

__device__ __forceinline__ float tf32_round(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// A_r split: hi/lo [batch][M][Kp], real view of the complex block A [M][K];
// grid-stride over output pairs (one complex element -> two floats)
__global__ void split_a_kernel(int batch, int M, int K, int Kp, const float2 *__restrict__ A, long long lda,
                               long long sa, float2 *__restrict__ hi, float2 *__restrict__ lo)
{
    const int kh = Kp / 2;                              // complex columns incl. padding
    const long long total = (long long)batch * M * kh;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(i % kh);
        const long long bm = i / kh;
        const int m = (int)(bm % M), b = (int)(bm / M);
        const float2 a = (k < K) ? A[(size_t)b * sa + (size_t)m * lda + k] : make_float2(0.f, 0.f);
        const float2 h = make_float2(tf32_round(a.x), tf32_round(a.y));
        hi[i] = h;
        lo[i] = make_float2(a.x - h.x, a.y - h.y);
    }
}

// Bt split: hi/lo [batch][2N][Kp], Bt[2n+r][2k+c] = [[Br, -Bi], [Bi, Br]][r][c];
// 32 x 32 complex tiles transposed through shared memory (coalesced both ways)
__global__ void __launch_bounds__(256)
split_b_kernel(int K, int N, int Kp, const float2 *__restrict__ B, long long ldb, long long sb,
               float *__restrict__ hi, float *__restrict__ lo)
{
    __shared__ float2 t[32][33];
    const int n0 = blockIdx.x * 32, k0 = blockIdx.y * 32, b = blockIdx.z;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;          // 32 x 8
    for (int r = ty; r < 32; r += 8) {
        const int k = k0 + r, n = n0 + tx;
        t[r][tx] = (k < K && n < N) ? B[(size_t)b * sb + (size_t)k * ldb + n] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    // output rows 2n + rr (64 per tile), columns 2k + c (64 per tile)
    for (int q = threadIdx.x; q < 64 * 64; q += 256) {
        const int orow = q / 64, ocol = q % 64;
        const int n = n0 + orow / 2, rr = orow & 1;
        const int kc = k0 * 2 + ocol;
        if (n >= N || kc >= Kp) continue;
        const float2 x = t[ocol / 2][orow / 2];
        const int c = ocol & 1;
        const float v = (rr == 0) ? (c == 0 ? x.x : -x.y) : (c == 0 ? x.y : x.x);
        const float h = tf32_round(v);
        const size_t o = ((size_t)b * 2 * N + 2 * n + rr) * Kp + kc;
        hi[o] = h;
        lo[o] = v - h;
    }
}

// (register cap of two CTAs per SM: one CTA fits by shared memory, and the
// cap leaves room for the LU panel kernel to run beside it)
__global__ void __launch_bounds__(TC_THREADS, 2)
tc_update_kernel(const __grid_constant__ CUtensorMap map_ahi, const __grid_constant__ CUtensorMap map_alo,
                 const __grid_constant__ CUtensorMap map_bhi, const __grid_constant__ CUtensorMap map_blo,
                 const __grid_constant__ CUtensorMap map_c, int use_tma_c,
                 int M, int Nr, int Kp, int tiles_n, int tiles_m, int batch, float *__restrict__ C,
                 long long ldc_r, long long sc_r, int *__restrict__ err, long long wait_limit)
{
    extern __shared__ unsigned char smem_raw[];
    TcSmem &s = *reinterpret_cast<TcSmem *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nst = Kp / BK;
    const int per_b = tiles_n * tiles_m;
    const int ntiles = per_b * batch;
    volatile int *failed = &s.failed;

    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(&s.tmem_base)), "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < STAGES; ++i) { mbar_init(&s.full[i], 1); mbar_init(&s.empty[i], 1); }
        for (int i = 0; i < 2; ++i) { mbar_init(&s.tfull[i], 1); mbar_init(&s.tempty[i], 4); }
        mbar_init(&s.drain, 1);
        s.failed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s.tmem_base;

    if (warp == 0 && lane == 0) {
        // ---- TMA producer: stage g % STAGES, its u-th use waits for the
        // MMAs of use u - 1 (empty phase u - 1)
        const uint32_t bytes = 4u * TILE_FLOATS * 4u;
        uint32_t g = 0;
        for (int t = blockIdx.x; t < ntiles && !*failed; t += gridDim.x) {
            const int b = t / per_b, r = t % per_b;
            const int m0 = (r / tiles_n) * BM, n0 = (r % tiles_n) * BNR;
            for (int ks = 0; ks < nst; ++ks, ++g) {
                const uint32_t st = g % STAGES, u = g / STAGES;
                if (u > 0 && !mbar_wait(&s.empty[st], (u - 1) & 1u, wait_limit)) {
                    *failed = 1;
                    break;
                }
                mbar_expect_tx(&s.full[st], bytes);
                tma_load_3d(s.a_hi[st], &map_ahi, ks * BK, m0, b, &s.full[st]);
                tma_load_3d(s.a_lo[st], &map_alo, ks * BK, m0, b, &s.full[st]);
                tma_load_3d(s.b_hi[st], &map_bhi, ks * BK, n0, b, &s.full[st]);
                tma_load_3d(s.b_lo[st], &map_blo, ks * BK, n0, b, &s.full[st]);
            }
        }
        {
            // the copies still in flight land before the CTA exits (on the normal
            // path they all have: each wait returns at once); the drain keeps the
            // long limit whatever the pipeline waits use
            const uint32_t j0 = g > STAGES ? g - STAGES : 0;
            for (uint32_t j = j0; j < g; ++j) mbar_wait(&s.full[j % STAGES], (j / STAGES) & 1u);
        }
    } else if (warp == 1 && lane == 0) {
        // ---- MMA issuer: tile i accumulates into TMEM buffer i & 1
        uint32_t g = 0;
        int i = 0;
        bool issued = false;
        for (int t = blockIdx.x; t < ntiles && !*failed; t += gridDim.x, ++i) {
            const uint32_t ab = i & 1, ui = i >> 1;
            if (ui > 0 && !mbar_wait(&s.tempty[ab], (ui - 1) & 1u, wait_limit)) { *failed = 1; break; }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t d = tmem + ab * BNR;
            for (int ks = 0; ks < nst; ++ks, ++g) {
                const uint32_t st = g % STAGES, u = g / STAGES;
                if (!mbar_wait(&s.full[st], u & 1u, wait_limit)) { *failed = 1; break; }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t ah = smem_u32(s.a_hi[st]), al = smem_u32(s.a_lo[st]);
                const uint32_t bh = smem_u32(s.b_hi[st]), bl = smem_u32(s.b_lo[st]);
#pragma unroll
                for (int kk = 0; kk < BK / 8; ++kk) {          // 8 tf32 = 32 bytes per MMA
                    const uint32_t off = kk * 32;
                    const uint32_t acc0 = (ks > 0 || kk > 0) ? 1u : 0u;
                    umma_tf32(d, umma_desc_sw128(ah + off), umma_desc_sw128(bh + off), acc0);
                    umma_tf32(d, umma_desc_sw128(ah + off), umma_desc_sw128(bl + off), 1u);
                    umma_tf32(d, umma_desc_sw128(al + off), umma_desc_sw128(bh + off), 1u);
                }
                issued = true;
                umma_commit(&s.empty[st]);
            }
            if (*failed) break;
            umma_commit(&s.tfull[ab]);
        }
        if (*failed && issued) {
            // the accumulators are released only after the MMAs in flight
            umma_commit(&s.drain);
            mbar_wait(&s.drain, 0);
        }
    } else if (warp >= 2) {
        // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows of
        // the tile), 32 columns at a time.
        //  TMA path: -acc is staged in shared memory (swizzled like the C
        //  tensor map) and added to C by a TMA reduce-add, so the epilogue
        //  issues no global loads; two staging boxes per warp alternate.
        //  Load/store path (C not 16-byte aligned): each slice is transposed
        //  through shared memory so the read-modify-write of C covers one
        //  128-byte row segment per instruction, and each lane prefetches its
        //  row of the next tile into L2 while that tile's MMAs run.
        const int q = warp & 3;
        auto prefetch_c = [&](int t) {
            if (use_tma_c || t >= ntiles) return;
            const int b = t / per_b, r = t % per_b;
            const int row = (r / tiles_n) * BM + q * 32 + lane, n0 = (r % tiles_n) * BNR;
            if (row >= M) return;
            const float *rp = C + (size_t)b * sc_r + (size_t)row * ldc_r;
            for (int c = n0; c < min(n0 + BNR, Nr); c += 32)
                asm volatile("prefetch.global.L2 [%0];" ::"l"(rp + c));
        };
        prefetch_c(blockIdx.x);
        int i = 0, nbox = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
            prefetch_c(t + gridDim.x);
            const int stop = __shfl_sync(0xffffffffu, *failed, 0);
            if (stop) break;
            const uint32_t ab = i & 1, ui = i >> 1;
            const bool ok = __all_sync(0xffffffffu, mbar_wait(&s.tfull[ab], ui & 1u, wait_limit));
            if (!ok) {
                if (lane == 0) *failed = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int b = t / per_b, r = t % per_b;
            const int m0 = (r / tiles_n) * BM, n0 = (r % tiles_n) * BNR;
            const int rows = min(32, M - (m0 + q * 32));
#pragma unroll 1
            for (int c32 = 0; c32 < BNR / 32; ++c32) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + ab * BNR + (uint32_t)(c32 * 32), v);
                if (use_tma_c) {
                    if (n0 + c32 * 32 >= Nr || rows <= 0) continue;
                    float *box = s.ep[q][nbox & 1];
                    // the reduce issued from this box two boxes ago has read it
                    if (lane == 0) asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                    __syncwarp();
#pragma unroll
                    for (int j4 = 0; j4 < 8; ++j4)
                        *reinterpret_cast<float4 *>(box + lane * 32 + ((j4 ^ (lane & 7)) << 2)) =
                            make_float4(-v[4 * j4], -v[4 * j4 + 1], -v[4 * j4 + 2], -v[4 * j4 + 3]);
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    __syncwarp();
                    if (lane == 0) {
                        asm volatile("cp.reduce.async.bulk.tensor.3d.global.shared::cta.add.tile.bulk_group"
                                     " [%0, {%1, %2, %3}], [%4];"
                                     ::"l"(reinterpret_cast<uint64_t>(&map_c)), "r"(n0 + c32 * 32),
                                       "r"(m0 + q * 32), "r"(b), "r"(smem_u32(box))
                                     : "memory");
                        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                    }
                    ++nbox;
                } else {
                    float(*tr)[33] = reinterpret_cast<float(*)[33]>(s.ep[q][0]);
#pragma unroll
                    for (int j = 0; j < 32; ++j) tr[lane][j] = v[j];
                    __syncwarp();
                    const int col = n0 + c32 * 32 + lane;
                    float *cb = C + (size_t)b * sc_r + (size_t)(m0 + q * 32) * ldc_r + col;
                    if (col < Nr && rows > 0) {
                        // all loads first (the compiler cannot reorder C loads past C stores)
                        float cv[32];
#pragma unroll
                        for (int j = 0; j < 32; ++j) cv[j] = (j < rows) ? cb[(size_t)j * ldc_r] : 0.f;
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            if (j < rows) cb[(size_t)j * ldc_r] = cv[j] - tr[j][lane];
                    }
                    __syncwarp();
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            if (lane == 0) mbar_arrive(&s.tempty[ab]);          // accumulator free for tile i + 2
        }
        // every reduce-add has completed before the kernel ends
        if (use_tma_c && lane == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0 && *failed) atomicExch(err, 1);
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// K-major [batch][rows][Kp] FP32 operand, box 32 x 128, 128-byte swizzle
bool make_map(CUtensorMap *map, const float *base, int rows, int Kp, int batch)
{
    auto enc = get_encode();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)batch};
    const cuuint64_t strides[2] = {(cuuint64_t)Kp * 4, (cuuint64_t)rows * Kp * 4};
    const cuuint32_t box[3] = {BK, BM, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// C [batch][M][Nr] FP32 (real view of the complex output), box 32 x 32, 128-byte
// swizzle, for the reduce-add epilogue; false when C's base or strides are not
// 16-byte multiples (the kernel then reads and writes C itself)
bool make_map_c(CUtensorMap *map, float *C, int M, int Nr, int batch, long long ldc_r, long long sc_r)
{
    if ((reinterpret_cast<uintptr_t>(C) & 15) || (ldc_r & 3) || (batch > 1 && (sc_r & 3))) return false;
    auto enc = get_encode();
    if (!enc) return false;
    const long long bstride = batch > 1 ? sc_r : (long long)M * ldc_r + ((4 - ((long long)M * ldc_r) % 4) % 4);
    const cuuint64_t dims[3] = {(cuuint64_t)Nr, (cuuint64_t)M, (cuuint64_t)batch};
    const cuuint64_t strides[2] = {(cuuint64_t)ldc_r * 4, (cuuint64_t)bstride * 4};
    const cuuint32_t box[3] = {32, 32, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, C, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

// Workspace layout: [0, 256) error flag (int, sticky: set to 1 by any call
// whose bounded in-kernel wait gave up; the caller clears it), then the split
// operands at a 256-byte boundary.
long long tc_update_workspace(int batch, int M, int N, int K)
{
    const long long Kp = ((2LL * K + BK - 1) / BK) * BK;
    return 4LL * Kp * batch * (2LL * M + 2LL * 2 * N) + 512;
}

// C[b] (M x N complex float) -= A[b] (M x K) B[b] (K x N) on the tensor cores.
// The sticky error flag at the start of the workspace is set if a bounded wait
// inside the kernel gave up (that tile is then left unchanged).
int tc_update(int batch, int M, int N, int K, const float2 *A, long long lda, long long sa,
              const float2 *B, long long ldb, long long sb, float2 *C, long long ldc, long long sc,
              void *work, cudaStream_t st)
{
    if (M <= 0 || N <= 0 || K <= 0) return GHOST_BOR_OK;
    const int Kp = ((2 * K + BK - 1) / BK) * BK;
    int *err = reinterpret_cast<int *>(work);
    float *w = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(work) + 256);
    float *ahi = w, *alo = ahi + (size_t)batch * M * Kp;
    float *bhi = alo + (size_t)batch * M * Kp, *blo = bhi + (size_t)batch * 2 * N * Kp;
    {
        const long long pairs = (long long)batch * M * (Kp / 2);
        const int blocks = (int)((pairs + 255) / 256 < 152 * 16 ? (pairs + 255) / 256 : 152 * 16);
        split_a_kernel<<<blocks, 256, 0, st>>>(batch, M, K, Kp, A, lda, sa, reinterpret_cast<float2 *>(ahi),
                                               reinterpret_cast<float2 *>(alo));
        int rc = check_launch("tc_update: split A");
        if (rc) return rc;
        dim3 g2((N + 31) / 32, (Kp / 2 + 31) / 32, batch);
        split_b_kernel<<<g2, 256, 0, st>>>(K, N, Kp, B, ldb, sb, bhi, blo);
        if ((rc = check_launch("tc_update: split B"))) return rc;
    }
    CUtensorMap mah, mal, mbh, mbl;
    if (!make_map(&mah, ahi, M, Kp, batch) || !make_map(&mal, alo, M, Kp, batch) ||
        !make_map(&mbh, bhi, 2 * N, Kp, batch) || !make_map(&mbl, blo, 2 * N, Kp, batch)) {
        set_last_error("tc_update: cuTensorMapEncodeTiled failed");
        return GHOST_BOR_ECUDA;
    }
    const size_t smem = sizeof(TcSmem) + 1024;
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(tc_update_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
            cudaSuccess)
            return check_launch("tc_update: smem attribute");
        attr = true;
    }
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
            sms = 1;
    }
    const int tiles_n = (2 * N + BNR - 1) / BNR, tiles_m = (M + BM - 1) / BM;
    const long long ntiles = (long long)tiles_n * tiles_m * batch;
    if (ntiles > 0x7fffffffLL) return GHOST_BOR_EUNSUPPORTED;
    const int grid = (int)(ntiles < sms ? ntiles : sms);      // persistent: one CTA per SM
    CUtensorMap mc;
    float *Cr = reinterpret_cast<float *>(C);
    const int use_tma_c = make_map_c(&mc, Cr, M, 2 * N, batch, 2 * ldc, 2 * sc) ? 1 : 0;
    if (!use_tma_c) mc = mah;                                   // unused by the kernel
    tc_update_kernel<<<grid, TC_THREADS, smem, st>>>(mah, mal, mbh, mbl, mc, use_tma_c, M, 2 * N, Kp, tiles_n,
                                                     tiles_m, batch, Cr, 2 * ldc, 2 * sc, err,
                                                     __atomic_load_n(&g_pipeline_wait_limit, __ATOMIC_RELAXED));
    return check_launch("tc_update");
}

}  // namespace gb

extern "C" void ghost_bor_set_wait_limit(long long polls)
{
    __atomic_store_n(&gb::g_pipeline_wait_limit, polls < 0 ? gb::WAIT_LIMIT : polls, __ATOMIC_RELAXED);
}

extern "C" long long ghost_bor_cgemm_tc_workspace(int batch, int M, int N, int K)
{
    return gb::tc_update_workspace(batch, M, N, K);
}

extern "C" int ghost_bor_cgemm_tc(int batch, int M, int N, int K,
                                  const void *A, long long lda, long long stride_a,
                                  const void *B, long long ldb, long long stride_b,
                                  void *C, long long ldc, long long stride_c,
                                  void *work, int *status, void *stream)
{
    if (batch < 1 || M < 0 || N < 0 || K < 0 || !A || !B || !C || !work || lda < K || ldb < N || ldc < N ||
        (reinterpret_cast<uintptr_t>(work) & 255))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(work, 0, sizeof(int), st) != cudaSuccess) return gb::check_launch("cgemm_tc: memset");
    const int rc = gb::tc_update(batch, M, N, K, reinterpret_cast<const float2 *>(A), lda, stride_a,
                                 reinterpret_cast<const float2 *>(B), ldb, stride_b,
                                 reinterpret_cast<float2 *>(C), ldc, stride_c, work, st);
    if (rc == GHOST_BOR_OK && status) {
        if (cudaMemcpyAsync(status, work, sizeof(int), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
            return gb::check_launch("cgemm_tc: status copy");
    }
    return rc;
}
