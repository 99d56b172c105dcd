// lu.cu -- batched dense complex LU with partial pivoting, triangular solves,
// mixed-precision residuals and small matrix helpers.  Replaces the LAPACK
// zgesv behind np.linalg.solve (bor_solver.py:753) and its residual
// (bor_solver.py:754-756) for every azimuthal mode at once.
//
// Right-looking blocked LU per matrix (one batch entry per mode):
//   panel   one CTA per matrix factors an NB-wide column panel (pivot search
//           with the LAPACK izamax rule |re| + |im|, first maximum wins)
//   laswp   row interchanges applied to the columns outside the panel
//   trsm    U12 = L11^-1 A12, one thread per column, L11 in shared memory
//   update  A22 -= L21 U12 (complex rank-NB update): the tcgen05 3xTF32 GEMM
//           of tc_gemm.cu when a workspace is given (FP32), else 64 x 64 SIMT
//           tiles
// with one step of look-ahead (the next panel overlaps the rest of the update
// on a side stream).  The same trsm/update kernels run the forward/back
// substitutions, in 256-row outer blocks on the tensor-core path.
#include "common.cuh"

namespace gb {

long long tc_update_workspace(int batch, int M, int N, int K);
int tc_update(int batch, int M, int N, int K, const float2 *A, long long lda, long long sa,
              const float2 *B, long long ldb, long long sb, float2 *C, long long ldc, long long sc,
              void *work, cudaStream_t st);

namespace {

template <class R> struct LuCfg;
template <> struct LuCfg<float> { static constexpr int NB = 64; };
template <> struct LuCfg<double> { static constexpr int NB = 32; };

constexpr int PANEL_THREADS = 512;
constexpr int kSolveBlocks = 4;      // tensor-core substitutions: outer blocks of 4 NB rows
constexpr int GT = 64;               // gemm tile (rows and columns)

// ---------------------------------------------------------------------------
// panel factorisation (one CTA per batch matrix)
// ---------------------------------------------------------------------------
// (register cap of two CTAs per SM, so that the panel of the next step fits
// beside the tensor-core update of the look-ahead LU)
template <class R>
__global__ void __launch_bounds__(PANEL_THREADS, 2)
panel_kernel(int n, int k0, int nb, C<R> *__restrict__ A, long long lda, long long sa,
             int *__restrict__ ipiv, int *__restrict__ info)
{
    using CT = C<R>;
    const int b = blockIdx.x;
    CT *Ab = A + (size_t)b * sa;
    int *piv = ipiv + (size_t)b * n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = PANEL_THREADS / 32;
    __shared__ R s_val[NW];
    __shared__ int s_idx[NW];
    __shared__ int s_piv;
    __shared__ CT s_prow[64];

    for (int jj = 0; jj < nb; ++jj) {
        const int col = k0 + jj;
        // --- pivot search: max |re|+|im|, smallest index on ties
        R best = R(-1);
        int bi = n;
        for (int i = col + tid; i < n; i += PANEL_THREADS) {
            const R v = cabs1(Ab[(size_t)i * lda + col]);
            if (v > best) { best = v; bi = i; }
        }
        for (int off = 16; off > 0; off >>= 1) {
            const R ov = __shfl_down_sync(0xffffffffu, best, off);
            const int oi = __shfl_down_sync(0xffffffffu, bi, off);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { s_val[warp] = best; s_idx[warp] = bi; }
        __syncthreads();
        if (warp == 0) {
            best = lane < NW ? s_val[lane] : R(-1);
            bi = lane < NW ? s_idx[lane] : n;
            for (int off = 16; off > 0; off >>= 1) {
                const R ov = __shfl_down_sync(0xffffffffu, best, off);
                const int oi = __shfl_down_sync(0xffffffffu, bi, off);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (lane == 0) {
                const int p = (bi < n) ? bi : col;
                s_piv = p;
                piv[col] = p;
                if (!(best > R(0)) && info[b] == 0) info[b] = col + 1;
            }
        }
        __syncthreads();
        const int p = s_piv;
        // --- swap rows col <-> p inside the panel columns
        if (p != col) {
            for (int c = k0 + tid; c < k0 + nb; c += PANEL_THREADS) {
                const CT t = Ab[(size_t)col * lda + c];
                Ab[(size_t)col * lda + c] = Ab[(size_t)p * lda + c];
                Ab[(size_t)p * lda + c] = t;
            }
        }
        __syncthreads();
        const CT pv = Ab[(size_t)col * lda + col];
        const int ncol = k0 + nb - col - 1;           // trailing panel columns
        for (int c = tid; c < ncol; c += PANEL_THREADS) s_prow[c] = Ab[(size_t)col * lda + col + 1 + c];
        __syncthreads();
        if (pv.x != R(0) || pv.y != R(0)) {
            // reciprocal of the pivot (LAPACK scales by 1/pivot)
            const R den = pv.x * pv.x + pv.y * pv.y;
            const CT inv = mk<R>(pv.x / den, -pv.y / den);
            // warps over groups of 32 rows, lanes over the trailing panel
            // columns; each warp loads the multipliers of its 32 rows at once
            // (one per lane), then all 32 row values of its column before the
            // first store, so a group costs one memory latency, not 32
            for (int i0 = col + 1 + 32 * warp; i0 < n; i0 += 32 * NW) {
                const int ir = i0 + lane;
                CT lmine = mk<R>(0, 0);
                if (ir < n) {
                    lmine = cmul(Ab[(size_t)ir * lda + col], inv);
                    Ab[(size_t)ir * lda + col] = lmine;
                }
                const int rows = min(32, n - i0);
                CT *rows0 = Ab + (size_t)i0 * lda + col + 1;
                for (int c0 = 0; c0 < ncol; c0 += 32) {
                    const int c = c0 + lane;
                    const bool act = c < ncol;
                    const CT u = act ? s_prow[c] : mk<R>(0, 0);
                    constexpr int QB = 8;                             // rows per batch of loads
#pragma unroll 1
                    for (int q0 = 0; q0 < 32; q0 += QB) {
                        CT v[QB];
#pragma unroll
                        for (int q = 0; q < QB; ++q)
                            if (act && q0 + q < rows) v[q] = rows0[(size_t)(q0 + q) * lda + c];
#pragma unroll
                        for (int q = 0; q < QB; ++q) {
                            CT l;
                            l.x = __shfl_sync(0xffffffffu, lmine.x, q0 + q);
                            l.y = __shfl_sync(0xffffffffu, lmine.y, q0 + q);
                            if (act && q0 + q < rows) rows0[(size_t)(q0 + q) * lda + c] = cfms(l, u, v[q]);
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// blocked panel factorisation, FP32 (one CTA per batch matrix): the panel is
// factored in sub-blocks of PW columns held in registers (each of the 256
// threads holds rows k0 + t + 256 s, s < RPT), so the pivot search, the row
// interchanges and the rank-1 updates of a sub-block touch no memory; the
// sub-block is then written back, its interchanges are applied to the other
// panel columns, and the rest of the panel gets one rank-PW update
// (U12 = L11^-1 A12, A22 -= L21 U12) -- one pass over it per sub-block instead
// of one per column.  Same pivots (LAPACK izamax rule) as panel_kernel.
// ---------------------------------------------------------------------------
constexpr int PB_THREADS = 256;
template <int RPT, int PW>    // rows per thread, columns per sub-block
__global__ void __launch_bounds__(PB_THREADS, 2)
panel_blocked_kernel(int n, int k0, int nb, float2 *__restrict__ A, long long lda, long long sa,
                     int *__restrict__ ipiv, int *__restrict__ info)
{
    using CT = float2;
    const int b = blockIdx.x;
    CT *Ab = A + (size_t)b * sa;
    int *piv = ipiv + (size_t)b * n;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = PB_THREADS / 32;
    __shared__ float s_val[NW];
    __shared__ int s_idx[NW];
    __shared__ int s_piv;
    __shared__ CT s_rowp[PW], s_rowc[PW];
    __shared__ CT s_l11[PW][PW];
    __shared__ CT s_u12[PW][64];

    for (int c0 = k0; c0 < k0 + nb; c0 += PW) {
        const int w = min(PW, k0 + nb - c0);
        CT blk[RPT][PW];
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
            const int i = k0 + tid + PB_THREADS * s;
#pragma unroll
            for (int q = 0; q < PW; ++q)
                blk[s][q] = (i < n && q < w) ? Ab[(size_t)i * lda + c0 + q] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int jj = 0; jj < PW; ++jj) {
            if (jj >= w) break;
            const int col = c0 + jj;
            // --- pivot search over rows >= col: max |re|+|im|, smallest index on ties
            float best = -1.f;
            int bi = n;
#pragma unroll
            for (int s = 0; s < RPT; ++s) {
                const int i = k0 + tid + PB_THREADS * s;
                if (i >= col && i < n) {
                    const float v = cabs1(blk[s][jj]);
                    if (v > best || (v == best && i < bi)) { best = v; bi = i; }
                }
            }
            for (int off = 16; off > 0; off >>= 1) {
                const float ov = __shfl_down_sync(0xffffffffu, best, off);
                const int oi = __shfl_down_sync(0xffffffffu, bi, off);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (lane == 0) { s_val[warp] = best; s_idx[warp] = bi; }
            __syncthreads();
            if (warp == 0) {
                best = lane < NW ? s_val[lane] : -1.f;
                bi = lane < NW ? s_idx[lane] : n;
                for (int off = 16; off > 0; off >>= 1) {
                    const float ov = __shfl_down_sync(0xffffffffu, best, off);
                    const int oi = __shfl_down_sync(0xffffffffu, bi, off);
                    if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
                }
                if (lane == 0) {
                    const int p = (bi < n) ? bi : col;
                    s_piv = p;
                    piv[col] = p;
                    if (!(best > 0.f) && info[b] == 0) info[b] = col + 1;
                }
            }
            __syncthreads();
            const int p = s_piv;
            // --- interchange rows col and p of the sub-block (through shared memory)
            const int oc = (col - k0) % PB_THREADS, sc = (col - k0) / PB_THREADS;
            const int op = (p - k0) % PB_THREADS, sp = (p - k0) / PB_THREADS;
#pragma unroll
            for (int s = 0; s < RPT; ++s) {
                if (tid == op && s == sp)
#pragma unroll
                    for (int q = 0; q < PW; ++q) s_rowp[q] = blk[s][q];
                if (tid == oc && s == sc)
#pragma unroll
                    for (int q = 0; q < PW; ++q) s_rowc[q] = blk[s][q];
            }
            __syncthreads();
            if (p != col) {
#pragma unroll
                for (int s = 0; s < RPT; ++s) {
                    if (tid == oc && s == sc)
#pragma unroll
                        for (int q = 0; q < PW; ++q) blk[s][q] = s_rowp[q];
                    if (tid == op && s == sp)
#pragma unroll
                        for (int q = 0; q < PW; ++q) blk[s][q] = s_rowc[q];
                }
            }
            // --- multipliers and the rank-1 update of the sub-block (pivot row = s_rowp)
            const CT pv = s_rowp[jj];
            if (pv.x != 0.f || pv.y != 0.f) {
                const float den = pv.x * pv.x + pv.y * pv.y;
                const CT inv = make_float2(pv.x / den, -pv.y / den);
#pragma unroll
                for (int s = 0; s < RPT; ++s) {
                    const int i = k0 + tid + PB_THREADS * s;
                    if (i > col && i < n) {
                        const CT l = cmul(blk[s][jj], inv);
                        blk[s][jj] = l;
#pragma unroll
                        for (int q = 0; q < PW; ++q)
                            if (q > jj && q < w) blk[s][q] = cfms(l, s_rowp[q], blk[s][q]);
                    }
                }
            }
            __syncthreads();                     // s_rowp / s_rowc are reused by the next column
        }
        // --- the sub-block back to memory; L11 to shared memory
#pragma unroll
        for (int s = 0; s < RPT; ++s) {
            const int i = k0 + tid + PB_THREADS * s;
            if (i < n)
#pragma unroll
                for (int q = 0; q < PW; ++q)
                    if (q < w) Ab[(size_t)i * lda + c0 + q] = blk[s][q];
            if (i >= c0 && i < c0 + w)
#pragma unroll
                for (int q = 0; q < PW; ++q) s_l11[i - c0][q] = blk[s][q];
        }
        __syncthreads();
        // --- the sub-block's interchanges on the panel's other columns, in order
        const int nother = nb - w;
        for (int jj = 0; jj < w; ++jj) {
            const int r = c0 + jj, pr = piv[r];
            if (pr != r)
                for (int t = tid; t < nother; t += PB_THREADS) {
                    const int c = k0 + (t < c0 - k0 ? t : t + w);
                    const CT x = Ab[(size_t)r * lda + c];
                    Ab[(size_t)r * lda + c] = Ab[(size_t)pr * lda + c];
                    Ab[(size_t)pr * lda + c] = x;
                }
            __syncthreads();
        }
        // --- rest of the panel: U12 = L11^-1 A12 (rows c0..c0+w-1), A22 -= L21 U12
        const int cr = c0 + w, ncol = k0 + nb - cr;
        if (ncol > 0) {
            for (int j = tid; j < ncol; j += PB_THREADS) {
                CT x[PW];
#pragma unroll
                for (int r = 0; r < PW; ++r) {
                    if (r < w) {
                        CT v = Ab[(size_t)(c0 + r) * lda + cr + j];
#pragma unroll
                        for (int q = 0; q < PW; ++q)
                            if (q < r) v = cfms(s_l11[r][q], x[q], v);
                        x[r] = v;
                        Ab[(size_t)(c0 + r) * lda + cr + j] = v;
                        s_u12[r][j] = v;
                    }
                }
            }
            __syncthreads();
            // warps over groups of 32 rows, lanes over the panel's remaining columns
            // (coalesced); each lane loads the PW multipliers of one row of the group
            // (the sub-block just written, L2-resident), and a batch of 8 rows' values
            // is loaded before the first store, so a batch costs one memory latency
            for (int i0 = cr + 32 * warp; i0 < n; i0 += 32 * NW) {
                const int ir = i0 + lane;
                CT lmine[PW];
#pragma unroll
                for (int q = 0; q < PW; ++q)
                    lmine[q] = (ir < n && q < w) ? Ab[(size_t)ir * lda + c0 + q] : make_float2(0.f, 0.f);
                const int rows = min(32, n - i0);
                CT *rows0 = Ab + (size_t)i0 * lda + cr;
                for (int jc = 0; jc < ncol; jc += 32) {
                    const int j = jc + lane;
                    const bool act = j < ncol;
                    CT u[PW];
#pragma unroll
                    for (int q = 0; q < PW; ++q) u[q] = act ? s_u12[q][j] : make_float2(0.f, 0.f);
                    constexpr int QB = RPT >= 12 ? 4 : 8;             // rows per batch of loads
#pragma unroll 1
                    for (int q0 = 0; q0 < 32; q0 += QB) {
                        CT v[QB];
#pragma unroll
                        for (int qq = 0; qq < QB; ++qq)
                            if (act && q0 + qq < rows) v[qq] = rows0[(size_t)(q0 + qq) * lda + j];
#pragma unroll
                        for (int qq = 0; qq < QB; ++qq) {
#pragma unroll
                            for (int q = 0; q < PW; ++q) {
                                CT l;
                                l.x = __shfl_sync(0xffffffffu, lmine[q].x, q0 + qq);
                                l.y = __shfl_sync(0xffffffffu, lmine[q].y, q0 + qq);
                                if (q < w) v[qq] = cfms(l, u[q], v[qq]);
                            }
                            if (act && q0 + qq < rows) rows0[(size_t)(q0 + qq) * lda + j] = v[qq];
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
}

// apply the panel's interchanges to the columns outside [k0, k0 + nb)
template <class R>
__global__ void laswp_kernel(int n, int k0, int nb, C<R> *__restrict__ A, long long lda, long long sa,
                             const int *__restrict__ ipiv)
{
    const int b = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ncols = n - nb;
    if (t >= ncols) return;
    const int c = (t < k0) ? t : t + nb;
    C<R> *Ab = A + (size_t)b * sa;
    const int *piv = ipiv + (size_t)b * n;
    for (int jj = 0; jj < nb; ++jj) {
        const int r = k0 + jj, p = piv[r];
        if (p != r) {
            const C<R> x = Ab[(size_t)r * lda + c];
            Ab[(size_t)r * lda + c] = Ab[(size_t)p * lda + c];
            Ab[(size_t)p * lda + c] = x;
        }
    }
}

// row interchanges of a right-hand-side block, all n pivots in order
template <class R>
__global__ void laswp_rhs_kernel(int n, int nrhs, C<R> *__restrict__ B, long long ldb, long long sb,
                                 const int *__restrict__ ipiv)
{
    const int b = blockIdx.y;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nrhs) return;
    C<R> *Bb = B + (size_t)b * sb;
    const int *piv = ipiv + (size_t)b * n;
    for (int r = 0; r < n; ++r) {
        const int p = piv[r];
        if (p != r) {
            const C<R> x = Bb[(size_t)r * ldb + c];
            Bb[(size_t)r * ldb + c] = Bb[(size_t)p * ldb + c];
            Bb[(size_t)p * ldb + c] = x;
        }
    }
}

// X := L^-1 X (unit lower) or U^-1 X (non-unit upper) for an nb-row block,
// one thread per column.  T points at the nb x nb diagonal block, held in
// shared memory; the thread's column of X is staged in shared memory too
// (column-per-thread layout, conflict-free), so the substitution is a short
// rolled loop instead of a fully unrolled NB x NB register program whose code
// would not fit the instruction cache.
constexpr int TRSM_COLS = 128;       // columns (threads) per CTA
template <class R, int NB, bool UPPER>
__global__ void __launch_bounds__(TRSM_COLS)
trsm_kernel(int nb, int ncols, const C<R> *__restrict__ T, long long ldt, long long st,
            C<R> *__restrict__ X, long long ldx, long long sx)
{
    using CT = C<R>;
    extern __shared__ __align__(16) unsigned char trsm_smem[];
    CT(*Ts)[NB + 1] = reinterpret_cast<CT(*)[NB + 1]>(trsm_smem);
    CT *Dinv = reinterpret_cast<CT *>(trsm_smem + sizeof(CT) * NB * (NB + 1));
    CT *Xs = Dinv + NB;                                   // [NB][TRSM_COLS]
    const int b = blockIdx.y;
    const CT *Tb = T + (size_t)b * st;
    for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) {
        const int r = i / nb, c = i % nb;
        Ts[r][c] = Tb[(size_t)r * ldt + c];
    }
    if (UPPER) {
        __syncthreads();
        for (int i = threadIdx.x; i < nb; i += blockDim.x) {
            const CT d = Ts[i][i];
            const R den = d.x * d.x + d.y * d.y;
            Dinv[i] = mk<R>(d.x / den, -d.y / den);
        }
    }
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = c < ncols;
    CT *Xb = X + (size_t)b * sx + c;
    CT *xs = Xs + threadIdx.x;
    for (int i = 0; i < nb; ++i) xs[i * TRSM_COLS] = act ? Xb[(size_t)i * ldx] : mk<R>(0, 0);
    __syncthreads();
    if (!act) return;
    // four partial sums per row keep four independent FMA chains (and their
    // shared-memory loads) in flight
    const CT z = mk<R>(0, 0);
    if (!UPPER) {
        for (int i = 1; i < nb; ++i) {
            CT s0 = xs[i * TRSM_COLS], s1 = z, s2 = z, s3 = z;
            int j = 0;
            for (; j + 3 < i; j += 4) {
                s0 = cfms(Ts[i][j], xs[j * TRSM_COLS], s0);
                s1 = cfms(Ts[i][j + 1], xs[(j + 1) * TRSM_COLS], s1);
                s2 = cfms(Ts[i][j + 2], xs[(j + 2) * TRSM_COLS], s2);
                s3 = cfms(Ts[i][j + 3], xs[(j + 3) * TRSM_COLS], s3);
            }
            for (; j < i; ++j) s0 = cfms(Ts[i][j], xs[j * TRSM_COLS], s0);
            xs[i * TRSM_COLS] = cadd(cadd(s0, s1), cadd(s2, s3));
        }
    } else {
        for (int i = nb - 1; i >= 0; --i) {
            CT s0 = xs[i * TRSM_COLS], s1 = z, s2 = z, s3 = z;
            int j = i + 1;
            for (; j + 3 < nb; j += 4) {
                s0 = cfms(Ts[i][j], xs[j * TRSM_COLS], s0);
                s1 = cfms(Ts[i][j + 1], xs[(j + 1) * TRSM_COLS], s1);
                s2 = cfms(Ts[i][j + 2], xs[(j + 2) * TRSM_COLS], s2);
                s3 = cfms(Ts[i][j + 3], xs[(j + 3) * TRSM_COLS], s3);
            }
            for (; j < nb; ++j) s0 = cfms(Ts[i][j], xs[j * TRSM_COLS], s0);
            xs[i * TRSM_COLS] = cmul(cadd(cadd(s0, s1), cadd(s2, s3)), Dinv[i]);
        }
    }
    for (int i = 0; i < nb; ++i) Xb[(size_t)i * ldx] = xs[i * TRSM_COLS];
}

template <class R, int NB>
constexpr size_t trsm_smem_bytes()
{
    return sizeof(C<R>) * ((size_t)NB * (NB + 1) + NB + (size_t)NB * TRSM_COLS);
}

// launch helper: one thread per column, TRSM_COLS columns per CTA
template <class R, int NB, bool UPPER>
int trsm_launch(int batch, int nb, int ncols, const C<R> *T, long long ldt, long long st, C<R> *X, long long ldx,
                long long sx, cudaStream_t s)
{
    constexpr size_t smem = trsm_smem_bytes<R, NB>();
    static bool attr = false;
    if (!attr) {
        if (cudaFuncSetAttribute(trsm_kernel<R, NB, UPPER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return check_launch("trsm: smem attribute");
        attr = true;
    }
    dim3 g((ncols + TRSM_COLS - 1) / TRSM_COLS, batch);
    trsm_kernel<R, NB, UPPER><<<g, TRSM_COLS, smem, s>>>(nb, ncols, T, ldt, st, X, ldx, sx);
    return check_launch(UPPER ? "trsm U" : "trsm L");
}

// C -= A B,  A: rows x K, B: K x cols, K <= NB; 64 x 64 tiles, 4 x 4 per thread
template <class R, int NB>
__global__ void __launch_bounds__(256)
gemm_update_kernel(int rows, int cols, int K,
                   const C<R> *__restrict__ A, long long lda, long long sa,
                   const C<R> *__restrict__ B, long long ldb, long long sb,
                   C<R> *__restrict__ Cm, long long ldc, long long sc)
{
    using CT = C<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CT *As = reinterpret_cast<CT *>(smem_raw);            // [GT][NB+1]
    CT *Bs = As + GT * (NB + 1);                          // [NB][GT]
    const int b = blockIdx.z;
    const int r0 = blockIdx.y * GT, c0 = blockIdx.x * GT;
    const CT *Ab = A + (size_t)b * sa;
    const CT *Bb = B + (size_t)b * sb;
    CT *Cb = Cm + (size_t)b * sc;
    const int tid = threadIdx.x;
    for (int i = tid; i < GT * K; i += 256) {
        const int r = i / K, kk = i % K;
        As[r * (NB + 1) + kk] = (r0 + r < rows) ? Ab[(size_t)(r0 + r) * lda + kk] : mk<R>(0, 0);
    }
    for (int i = tid; i < K * GT; i += 256) {
        const int kk = i / GT, c = i % GT;
        Bs[kk * GT + c] = (c0 + c < cols) ? Bb[(size_t)kk * ldb + c0 + c] : mk<R>(0, 0);
    }
    __syncthreads();
    const int ty = tid >> 4, tx = tid & 15;
    CT acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = mk<R>(0, 0);
    for (int kk = 0; kk < K; ++kk) {
        CT a[4], bv[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[(ty + 16 * i) * (NB + 1) + kk];
#pragma unroll
        for (int j = 0; j < 4; ++j) bv[j] = Bs[kk * GT + tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = cfma(a[i], bv[j], acc[i][j]);
    }
    // all loads of C first, then the stores (keeps 16 loads in flight)
    CT cv[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = r0 + ty + 16 * i;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = c0 + tx + 16 * j;
            cv[i][j] = (r < rows && c < cols) ? Cb[(size_t)r * ldc + c] : mk<R>(0, 0);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = r0 + ty + 16 * i;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = c0 + tx + 16 * j;
            if (r < rows && c < cols) Cb[(size_t)r * ldc + c] = csub(cv[i][j], acc[i][j]);
        }
    }
}

template <class R>
int gemm_update(int batch, int rows, int cols, int K, const C<R> *A, long long lda, long long sa,
                const C<R> *B, long long ldb, long long sb, C<R> *Cm, long long ldc, long long sc,
                cudaStream_t st)
{
    if (rows <= 0 || cols <= 0 || K <= 0) return GHOST_BOR_OK;
    constexpr int NB = LuCfg<R>::NB;
    const size_t smem = sizeof(C<R>) * ((size_t)GT * (NB + 1) + (size_t)NB * GT);
    static bool attr_set = false;
    if (!attr_set) {
        if (cudaFuncSetAttribute(gemm_update_kernel<R, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess)
            return check_launch("gemm_update: smem attribute");
        attr_set = true;
    }
    dim3 grid((cols + GT - 1) / GT, (rows + GT - 1) / GT, batch);
    gemm_update_kernel<R, NB><<<grid, 256, smem, st>>>(rows, cols, K, A, lda, sa, B, ldb, sb, Cm, ldc, sc);
    return check_launch("gemm_update");
}

// C -= A B: tensor cores (3xTF32) for FP32 when a workspace is given, SIMT otherwise
template <class R>
int update(int batch, int rows, int cols, int K, const C<R> *A, long long lda, long long sa,
           const C<R> *B, long long ldb, long long sb, C<R> *Cm, long long ldc, long long sc,
           void *work, cudaStream_t st)
{
    if constexpr (sizeof(R) == 4) {
        if (work)
            return tc_update(batch, rows, cols, K, A, lda, sa, B, ldb, sb, Cm, ldc, sc, work, st);
    }
    return gemm_update<R>(batch, rows, cols, K, A, lda, sa, B, ldb, sb, Cm, ldc, sc, st);
}

// Side stream (higher priority for the panel on the caller's stream is not
// needed: the panel is launched first) and events of the look-ahead LU, one
// set per device, created on first use.
struct LookAhead {
    cudaStream_t side = nullptr;
    cudaEvent_t la = nullptr, rest = nullptr;
};

bool look_ahead(LookAhead &L)
{
    static thread_local LookAhead cache[16];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) return false;
    LookAhead &c = cache[dev];
    if (!c.side) {
        if (cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking) != cudaSuccess) return false;
        if (cudaEventCreateWithFlags(&c.la, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&c.rest, cudaEventDisableTiming) != cudaSuccess)
            return false;
    }
    L = c;
    return true;
}

// the panel of one step: the register-blocked FP32 kernel while its rows fit
// (n - k0 <= 256 x 24 rows; sub-blocks of 4 columns up to 3072 rows, of 2
// above), else the column-by-column kernel
template <class R>
int panel_launch(int batch, int n, int k0, int nb, C<R> *A, long long lda, long long sa, int *ipiv, int *info,
                 cudaStream_t st)
{
    if constexpr (sizeof(R) == 4) {
        const int rows = n - k0;
        if (nb <= 64 && rows <= PB_THREADS * 24) {
            if (rows <= PB_THREADS * 4)
                panel_blocked_kernel<4, 4><<<batch, PB_THREADS, 0, st>>>(n, k0, nb, A, lda, sa, ipiv, info);
            else if (rows <= PB_THREADS * 8)
                panel_blocked_kernel<8, 4><<<batch, PB_THREADS, 0, st>>>(n, k0, nb, A, lda, sa, ipiv, info);
            else if (rows <= PB_THREADS * 12)
                panel_blocked_kernel<12, 4><<<batch, PB_THREADS, 0, st>>>(n, k0, nb, A, lda, sa, ipiv, info);
            else if (rows <= PB_THREADS * 16)
                panel_blocked_kernel<16, 2><<<batch, PB_THREADS, 0, st>>>(n, k0, nb, A, lda, sa, ipiv, info);
            else
                panel_blocked_kernel<24, 2><<<batch, PB_THREADS, 0, st>>>(n, k0, nb, A, lda, sa, ipiv, info);
            return check_launch("getrf: blocked panel");
        }
    }
    panel_kernel<R><<<batch, PANEL_THREADS, 0, st>>>(n, k0, nb, A, lda, sa, ipiv, info);
    return check_launch("getrf: panel");
}

// Right-looking blocked LU with one step of look-ahead: the trailing update of
// step k is split into the next panel's NB columns (caller's stream) and the
// remaining columns (side stream), so the panel of step k + 1 -- a
// latency-bound kernel with one CTA per matrix -- runs while the bulk of the
// update of step k fills the other SMs.  The row swaps of step k + 1 touch
// every column and wait for the side stream first; the tensor-core workspace
// is used by one update at a time (the side update starts after the
// look-ahead update of its step and finishes before the next one starts).
template <class R>
int getrf_impl(int batch, int n, C<R> *A, long long lda, long long sa, int *ipiv, int *info, void *work,
               cudaStream_t st)
{
    constexpr int NB = LuCfg<R>::NB;
    if (cudaMemsetAsync(info, 0, sizeof(int) * batch, st) != cudaSuccess) return check_launch("getrf: memset");
    LookAhead L;
    const bool la = look_ahead(L);
    bool rest_pending = false;
    int rc;
    for (int k0 = 0; k0 < n; k0 += NB) {
        const int nb = min(NB, n - k0);
        if ((rc = panel_launch<R>(batch, n, k0, nb, A, lda, sa, ipiv, info, st))) return rc;
        if (rest_pending) {
            // the row swaps below touch the columns the side stream is updating
            if (cudaStreamWaitEvent(st, L.rest, 0) != cudaSuccess) return check_launch("getrf: wait");
            rest_pending = false;
        }
        if (n - nb > 0) {
            dim3 g((n - nb + 255) / 256, batch);
            laswp_kernel<R><<<g, 256, 0, st>>>(n, k0, nb, A, lda, sa, ipiv);
            if ((rc = check_launch("getrf: laswp"))) return rc;
        }
        const int rest = n - k0 - nb;
        if (rest > 0) {
            if ((rc = trsm_launch<R, NB, false>(batch, nb, rest, A + (size_t)k0 * lda + k0, lda, sa,
                                                A + (size_t)k0 * lda + k0 + nb, lda, sa, st)))
                return rc;
            const C<R> *L21 = A + (size_t)(k0 + nb) * lda + k0;
            const C<R> *U12 = A + (size_t)k0 * lda + k0 + nb;
            C<R> *A22 = A + (size_t)(k0 + nb) * lda + k0 + nb;
            const int ahead = min(NB, rest);                    // columns of the next panel
            if (!la || rest <= ahead) {
                if ((rc = update<R>(batch, rest, rest, nb, L21, lda, sa, U12, lda, sa, A22, lda, sa, work, st)))
                    return rc;
                continue;
            }
            if ((rc = update<R>(batch, rest, ahead, nb, L21, lda, sa, U12, lda, sa, A22, lda, sa, work, st)))
                return rc;
            if (cudaEventRecord(L.la, st) != cudaSuccess || cudaStreamWaitEvent(L.side, L.la, 0) != cudaSuccess)
                return check_launch("getrf: look-ahead event");
            if ((rc = update<R>(batch, rest, rest - ahead, nb, L21, lda, sa, U12 + ahead, lda, sa, A22 + ahead,
                                lda, sa, work, L.side)))
                return rc;
            if (cudaEventRecord(L.rest, L.side) != cudaSuccess) return check_launch("getrf: side event");
            rest_pending = true;
        }
    }
    if (rest_pending && cudaStreamWaitEvent(st, L.rest, 0) != cudaSuccess) return check_launch("getrf: final wait");
    return GHOST_BOR_OK;
}

template <class R>
int getrs_impl(int batch, int n, int nrhs, const C<R> *A, long long lda, long long sa, const int *ipiv,
               C<R> *B, long long ldb, long long sb, void *work, cudaStream_t st)
{
    constexpr int NB = LuCfg<R>::NB;
    {
        dim3 g((nrhs + 127) / 128, batch);
        laswp_rhs_kernel<R><<<g, 128, 0, st>>>(n, nrhs, B, ldb, sb, ipiv);
        int rc = check_launch("getrs: laswp");
        if (rc) return rc;
    }
    // The substitutions run in outer blocks of NBS rows: inside a block, NB-row
    // diagonal solves and updates of the block's remaining rows; then one
    // update of every row below (above) the block with K = NBS.  The large
    // updates read and write the right-hand sides once per NBS rows, so on the
    // tensor-core path (whose updates are bound by that traffic) NBS = 4 NB.
    const int NBS = (sizeof(R) == 4 && work) ? kSolveBlocks * NB : NB;
    int rc;
    for (int k0 = 0; k0 < n; k0 += NBS) {
        const int kb = min(NBS, n - k0);
        for (int j0 = k0; j0 < k0 + kb; j0 += NB) {
            const int nb = min(NB, k0 + kb - j0);
            if ((rc = trsm_launch<R, NB, false>(batch, nb, nrhs, A + (size_t)j0 * lda + j0, lda, sa,
                                                B + (size_t)j0 * ldb, ldb, sb, st)))
                return rc;
            if ((rc = update<R>(batch, k0 + kb - j0 - nb, nrhs, nb, A + (size_t)(j0 + nb) * lda + j0, lda, sa,
                                B + (size_t)j0 * ldb, ldb, sb, B + (size_t)(j0 + nb) * ldb, ldb, sb, work, st)))
                return rc;
        }
        if ((rc = update<R>(batch, n - k0 - kb, nrhs, kb, A + (size_t)(k0 + kb) * lda + k0, lda, sa,
                            B + (size_t)k0 * ldb, ldb, sb, B + (size_t)(k0 + kb) * ldb, ldb, sb, work, st)))
            return rc;
    }
    const int last = ((n - 1) / NBS) * NBS;
    for (int k0 = last; k0 >= 0; k0 -= NBS) {
        const int kb = min(NBS, n - k0);
        for (int j0 = k0 + ((kb - 1) / NB) * NB; j0 >= k0; j0 -= NB) {
            const int nb = min(NB, k0 + kb - j0);
            if ((rc = trsm_launch<R, NB, true>(batch, nb, nrhs, A + (size_t)j0 * lda + j0, lda, sa,
                                               B + (size_t)j0 * ldb, ldb, sb, st)))
                return rc;
            if ((rc = update<R>(batch, j0 - k0, nrhs, nb, A + (size_t)k0 * lda + j0, lda, sa,
                                B + (size_t)j0 * ldb, ldb, sb, B + (size_t)k0 * ldb, ldb, sb, work, st)))
                return rc;
        }
        if ((rc = update<R>(batch, k0, nrhs, kb, A + k0, lda, sa, B + (size_t)k0 * ldb, ldb, sb, B, ldb, sb,
                            work, st)))
            return rc;
    }
    return GHOST_BOR_OK;
}

// ---------------------------------------------------------------------------
// residuals
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool is_masked(const int *mr, int r)
{
    return mr[0] == r || mr[1] == r || mr[2] == r || mr[3] == r;
}

// R = B - Zf X - band X, all operands complex double.  64 x 64 tiles over
// (rows, rhs).  Zf and X are split into two FP32 words each (hi + lo, ~48
// bits); the hi*hi products are summed in FP32 over 4-term chunks and the
// chunk sums folded into a double-float (TwoSum) accumulator; the small
// hi*lo + lo*hi products and the TwoSum errors share one FP32 sum.  The FP64 band (near/self
// blocks) is applied in FP64.
constexpr int RK = 16;

__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float v)
{
    const float s = hi + v;
    const float bb = s - hi;
    lo += (hi - (s - bb)) + (v - bb);
    hi = s;
}

__device__ __forceinline__ void split2(double2 v, float2 &h, float2 &l)
{
    h = make_float2((float)v.x, (float)v.y);
    l = make_float2((float)(v.x - (double)h.x), (float)(v.y - (double)h.y));
}

// tile element loaders: Z as complex double (split on the fly) or as its
// pre-split FP32 words (hi.re, hi.im, lo.re, lo.im); X as complex double or as
// an FP32 solution (low word zero)
__device__ __forceinline__ float4 split_words(double2 v)
{
    float2 h, l;
    split2(v, h, l);
    return make_float4(h.x, h.y, l.x, l.y);
}
__device__ __forceinline__ float4 z_words(const double2 *p) { return split_words(*p); }
__device__ __forceinline__ float4 z_words(const float4 *p) { return *p; }
__device__ __forceinline__ float4 x_words(const double2 *p) { return split_words(*p); }
__device__ __forceinline__ float4 x_words(const float2 *p) { const float2 v = *p; return make_float4(v.x, v.y, 0.f, 0.f); }
__device__ __forceinline__ double2 ld_x(const double2 *p) { return *p; }
__device__ __forceinline__ double2 ld_x(const float2 *p) { const float2 v = *p; return make_double2(v.x, v.y); }

// XT = double2: X in FP64, split into two FP32 words like Z.
// XT = float2:  X is an FP32 solution, its low word is zero and the Z_hi X_lo
//               products are skipped.
// ZT = double2: Z_far in complex double, split while staging the tiles;
// ZT = float4:  Z_far already split in place (ghost_bor_split_words), so the
//               staging does no FP64 work.
template <class XT, class ZT>
__global__ void __launch_bounds__(256)
residual_mixed_kernel(int n, int nrhs, int Nn, const ZT *__restrict__ Zf, long long ldz, long long sz,
                      const double2 *__restrict__ band, const int *__restrict__ mask_rows,
                      const XT *__restrict__ X, const double2 *__restrict__ B, long long ldb, long long sbb,
                      double2 *__restrict__ R, float2 *__restrict__ Rlo, double *__restrict__ norms)
{
    constexpr bool kXlo = sizeof(XT) == sizeof(double2);
    // tiles hold both FP32 words of each complex value: (hi.re, hi.im, lo.re, lo.im)
    // Zs is transposed (Zs[k][row]) and padded by one float4 per k so that the
    // staging stores (consecutive threads -> consecutive k) hit distinct banks
    __shared__ float4 Zs[RK][GT + 1];
    __shared__ float4 Xs[RK][GT];
    double (*red)[8] = reinterpret_cast<double (*)[8]>(&Zs[0][0]);   // reused after the K loop
    const int b = blockIdx.z;
    const int r0 = blockIdx.y * GT, c0 = blockIdx.x * GT;
    const ZT *Zb = Zf + (size_t)b * sz;
    const XT *Xb = X + (size_t)b * sbb;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    // hi: leading sum of the hi*hi products; sm: low-order part (hi*lo + lo*hi
    // products and the rounding errors of the hi sums, captured by TwoSum)
    float2 hi[4][4], sm[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) { hi[i][j] = make_float2(0, 0); sm[i][j] = make_float2(0, 0); }

    // each thread stages 4 Z and 4 X elements per tile (GT * RK = 1024 each)
    float4 zp[4], xp[4];
    auto fetch = [&](int k0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = tid + 256 * q;
            const int r = i / RK, kk = i % RK;
            zp[q] = (r0 + r < n && k0 + kk < n) ? z_words(Zb + (size_t)(r0 + r) * ldz + k0 + kk)
                                                : make_float4(0.f, 0.f, 0.f, 0.f);
            const int kx = i / GT, c = i % GT;
            xp[q] = (k0 + kx < n && c0 + c < nrhs) ? x_words(Xb + (size_t)(k0 + kx) * ldb + c0 + c)
                                                   : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    auto stage = [&]() {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int i = tid + 256 * q;
            Zs[i % RK][i / RK] = zp[q];
            Xs[i / GT][i % GT] = xp[q];
        }
    };
    fetch(0);
    for (int k0 = 0; k0 < n; k0 += RK) {
        __syncthreads();                 // previous tile fully consumed
        stage();
        __syncthreads();
        if (k0 + RK < n) fetch(k0 + RK); // global loads overlap the math below
#pragma unroll 1
        for (int k4 = 0; k4 < RK; k4 += 4) {
            // FP32 partial sums over 4 k-steps, folded into (hi, sm) by TwoSum
            float2 ac[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) ac[i][j] = make_float2(0, 0);
#pragma unroll
            for (int kk = k4; kk < k4 + 4; ++kk) {
                float4 a[4], x[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = Zs[kk][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) x[j] = Xs[kk][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float2 ah = make_float2(a[i].x, a[i].y), al = make_float2(a[i].z, a[i].w);
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const float2 xh = make_float2(x[j].x, x[j].y), xl = make_float2(x[j].z, x[j].w);
                        ac[i][j] = cfma(ah, xh, ac[i][j]);
                        if constexpr (kXlo) sm[i][j] = cfma(ah, xl, sm[i][j]);
                        sm[i][j] = cfma(al, xh, sm[i][j]);
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    two_sum_acc(hi[i][j].x, sm[i][j].x, ac[i][j].x);
                    two_sum_acc(hi[i][j].y, sm[i][j].y, ac[i][j].y);
                }
        }
    }
    __syncthreads();                     // Zs is reused for the norm reduction below
    const int *mr = mask_rows + 4 * b;
    const double2 *Bb = B + (size_t)b * sbb;
    double rn = 0.0, bn = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = r0 + ty + 16 * i;
        if (r >= n) continue;
        const bool masked = is_masked(mr, r);
        const int half = r >= Nn ? 1 : 0, node = r - half * Nn;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = c0 + tx + 16 * j;
            if (c >= nrhs) continue;
            const double2 bv = Bb[(size_t)r * ldb + c];
            const double zx = (double)hi[i][j].x + (double)sm[i][j].x;
            const double zy = (double)hi[i][j].y + (double)sm[i][j].y;
            double2 rv = make_double2(bv.x - zx, bv.y - zy);
            if (band) {
                for (int ch = 0; ch < 2; ++ch) {
                    const double2 *bd = band + (((size_t)b * 4 + 2 * half + ch) * Nn + node) * 5;
                    for (int d = 0; d < 5; ++d) {
                        const int jn = node + d - 2;
                        if (jn < 0 || jn >= Nn) continue;
                        rv = cfms(bd[d], ld_x(Xb + (size_t)(ch * Nn + jn) * ldb + c), rv);
                    }
                }
            }
            if (masked) rv = make_double2(0, 0);
            if (R) R[(size_t)b * sbb + (size_t)r * ldb + c] = rv;
            if (Rlo) Rlo[(size_t)b * sbb + (size_t)r * ldb + c] = make_float2((float)rv.x, (float)rv.y);
            rn += rv.x * rv.x + rv.y * rv.y;
            bn += bv.x * bv.x + bv.y * bv.y;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        rn += __shfl_down_sync(0xffffffffu, rn, off);
        bn += __shfl_down_sync(0xffffffffu, bn, off);
    }
    if ((tid & 31) == 0) { red[0][tid >> 5] = rn; red[1][tid >> 5] = bn; }
    __syncthreads();
    if (tid == 0) {
        double a = 0, c = 0;
        for (int w = 0; w < 8; ++w) { a += red[0][w]; c += red[1][w]; }
        atomicAdd(norms + 2 * b, a);
        atomicAdd(norms + 2 * b + 1, c);
    }
}

constexpr int RK64 = 16;
__global__ void __launch_bounds__(256)
residual64_kernel(int n, int nrhs, const double2 *__restrict__ Z, long long ldz, long long sz,
                  const double2 *__restrict__ X, const double2 *__restrict__ B, long long ldb, long long sbb,
                  double2 *__restrict__ R, double *__restrict__ norms)
{
    __shared__ double2 Zs[GT][RK64 + 1];
    __shared__ double2 Xs[RK64][GT];
    __shared__ double red[2][8];
    const int b = blockIdx.z;
    const int r0 = blockIdx.y * GT, c0 = blockIdx.x * GT;
    const double2 *Zb = Z + (size_t)b * sz;
    const double2 *Xb = X + (size_t)b * sbb;
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    double2 acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = make_double2(0, 0);
    for (int k0 = 0; k0 < n; k0 += RK64) {
        __syncthreads();
        for (int i = tid; i < GT * RK64; i += 256) {
            const int r = i / RK64, kk = i % RK64;
            Zs[r][kk] = (r0 + r < n && k0 + kk < n) ? Zb[(size_t)(r0 + r) * ldz + k0 + kk] : make_double2(0, 0);
        }
        for (int i = tid; i < RK64 * GT; i += 256) {
            const int kk = i / GT, c = i % GT;
            Xs[kk][c] = (k0 + kk < n && c0 + c < nrhs) ? Xb[(size_t)(k0 + kk) * ldb + c0 + c] : make_double2(0, 0);
        }
        __syncthreads();
        for (int kk = 0; kk < RK64; ++kk) {
            double2 a[4], x[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = Zs[ty + 16 * i][kk];
#pragma unroll
            for (int j = 0; j < 4; ++j) x[j] = Xs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = cfma(a[i], x[j], acc[i][j]);
        }
    }
    const double2 *Bb = B + (size_t)b * sbb;
    double rn = 0.0, bn = 0.0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int r = r0 + ty + 16 * i;
        if (r >= n) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = c0 + tx + 16 * j;
            if (c >= nrhs) continue;
            const double2 bv = Bb[(size_t)r * ldb + c];
            const double2 rv = make_double2(bv.x - acc[i][j].x, bv.y - acc[i][j].y);
            if (R) R[(size_t)b * sbb + (size_t)r * ldb + c] = rv;
            rn += rv.x * rv.x + rv.y * rv.y;
            bn += bv.x * bv.x + bv.y * bv.y;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        rn += __shfl_down_sync(0xffffffffu, rn, off);
        bn += __shfl_down_sync(0xffffffffu, bn, off);
    }
    if ((tid & 31) == 0) { red[0][tid >> 5] = rn; red[1][tid >> 5] = bn; }
    __syncthreads();
    if (tid == 0) {
        double a = 0, c = 0;
        for (int w = 0; w < 8; ++w) { a += red[0][w]; c += red[1][w]; }
        atomicAdd(norms + 2 * b, a);
        atomicAdd(norms + 2 * b + 1, c);
    }
}

// ---------------------------------------------------------------------------
// compose / mask / convert
// ---------------------------------------------------------------------------
__global__ void compose_kernel(int n, int Nn, const double2 *__restrict__ Zf, long long ldz, long long sz,
                               const double2 *__restrict__ band, const int *__restrict__ mask_rows,
                               float2 *__restrict__ A, long long lda, long long sa)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    const int b = blockIdx.z;
    if (j >= n) return;
    const int *mr = mask_rows + 4 * b;
    float2 out;
    if (is_masked(mr, i) || is_masked(mr, j)) {
        out = make_float2(i == j ? 1.f : 0.f, 0.f);
    } else {
        double2 v = Zf[(size_t)b * sz + (size_t)i * ldz + j];
        if (band) {
            const int a = i >= Nn, ch = j >= Nn;
            const int ii = i - a * Nn, jj = j - ch * Nn;
            const int d = jj - ii + 2;
            if (d >= 0 && d <= 4) {
                const double2 bv = band[(((size_t)b * 4 + 2 * a + ch) * Nn + ii) * 5 + d];
                v.x += bv.x; v.y += bv.y;
            }
        }
        out = make_float2((float)v.x, (float)v.y);
    }
    A[(size_t)b * sa + (size_t)i * lda + j] = out;
}

__global__ void mask64_kernel(int n, const int *__restrict__ mask_rows, double2 *__restrict__ Z,
                              long long ldz, long long sz)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int slot = blockIdx.y;
    const int b = blockIdx.z;
    const int r = mask_rows[4 * b + slot];
    if (r < 0 || r >= n || t >= n) return;
    double2 *Zb = Z + (size_t)b * sz;
    const double2 v = make_double2(t == r ? 1.0 : 0.0, 0.0);
    Zb[(size_t)r * ldz + t] = v;
    Zb[(size_t)t * ldz + r] = v;
}

__global__ void convert_kernel(int dir, int rows, int cols, const void *__restrict__ src, long long lds,
                               long long ss, void *__restrict__ dst, long long ldd, long long sd)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    const int b = blockIdx.z;
    if (c >= cols) return;
    if (dir == 0) {
        const double2 v = reinterpret_cast<const double2 *>(src)[(size_t)b * ss + (size_t)r * lds + c];
        reinterpret_cast<float2 *>(dst)[(size_t)b * sd + (size_t)r * ldd + c] = make_float2((float)v.x, (float)v.y);
    } else if (dir == 3) {
        reinterpret_cast<float2 *>(dst)[(size_t)b * sd + (size_t)r * ldd + c] =
            reinterpret_cast<const float2 *>(src)[(size_t)b * ss + (size_t)r * lds + c];
    } else {
        const float2 v = reinterpret_cast<const float2 *>(src)[(size_t)b * ss + (size_t)r * lds + c];
        double2 *o = reinterpret_cast<double2 *>(dst) + (size_t)b * sd + (size_t)r * ldd + c;
        if (dir == 1) *o = make_double2(v.x, v.y);
        else { double2 t = *o; t.x += v.x; t.y += v.y; *o = t; }
    }
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" long long ghost_bor_getrf_workspace(int prec, int batch, int n)
{
    if (prec != GHOST_BOR_F32 || batch < 1 || n < 1) return 0;
    return tc_update_workspace(batch, n, n, LuCfg<float>::NB);
}

extern "C" long long ghost_bor_getrs_workspace(int prec, int batch, int n, int nrhs)
{
    if (prec != GHOST_BOR_F32 || batch < 1 || n < 1 || nrhs < 1) return 0;
    return tc_update_workspace(batch, n, nrhs, kSolveBlocks * LuCfg<float>::NB);
}

static bool tc_work_ok(const void *work)
{
    return !work || (reinterpret_cast<uintptr_t>(work) & 255) == 0;
}

extern "C" int ghost_bor_getrf(int prec, int batch, int n, void *A, long long lda, long long stride_a,
                               int *ipiv, int *info, void *work, void *stream)
{
    if (batch < 1 || n < 1 || !A || !ipiv || !info || lda < n || stride_a < lda * n || !tc_work_ok(work))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (prec == GHOST_BOR_F32) {
        if (work && cudaMemsetAsync(work, 0, sizeof(int), st) != cudaSuccess) return check_launch("getrf: memset");
        return getrf_impl<float>(batch, n, reinterpret_cast<float2 *>(A), lda, stride_a, ipiv, info, work, st);
    }
    if (prec == GHOST_BOR_F64)
        return getrf_impl<double>(batch, n, reinterpret_cast<double2 *>(A), lda, stride_a, ipiv, info, nullptr, st);
    return GHOST_BOR_EINVAL;
}

extern "C" int ghost_bor_getrs(int prec, int batch, int n, int nrhs,
                               const void *A, long long lda, long long stride_a, const int *ipiv,
                               void *B, long long ldb, long long stride_b, void *work, void *stream)
{
    if (batch < 1 || n < 1 || nrhs < 1 || !A || !ipiv || !B || lda < n || ldb < nrhs ||
        stride_a < lda * n || stride_b < ldb * n || !tc_work_ok(work))
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (prec == GHOST_BOR_F32) {
        if (work && cudaMemsetAsync(work, 0, sizeof(int), st) != cudaSuccess) return check_launch("getrs: memset");
        return getrs_impl<float>(batch, n, nrhs, reinterpret_cast<const float2 *>(A), lda, stride_a, ipiv,
                                 reinterpret_cast<float2 *>(B), ldb, stride_b, work, st);
    }
    if (prec == GHOST_BOR_F64)
        return getrs_impl<double>(batch, n, nrhs, reinterpret_cast<const double2 *>(A), lda, stride_a, ipiv,
                                  reinterpret_cast<double2 *>(B), ldb, stride_b, nullptr, st);
    return GHOST_BOR_EINVAL;
}

extern "C" int ghost_bor_residual(int batch, int n, int nrhs, int Nn,
                                  const void *Zf, long long ldz, long long stride_z,
                                  const double *band, const int *mask_rows,
                                  const double *X, const double *B, long long ldb, long long stride_b,
                                  double *R, float *Rlo, double *norms, void *stream)
{
    if (batch < 1 || n < 1 || nrhs < 1 || !Zf || !mask_rows || !X || !B || !R || !norms ||
        ldz < n || ldb < nrhs || n != 2 * Nn)
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(norms, 0, sizeof(double) * 2 * batch, st) != cudaSuccess) return check_launch("residual: memset");
    dim3 grid((nrhs + GT - 1) / GT, (n + GT - 1) / GT, batch);
    residual_mixed_kernel<double2, double2><<<grid, 256, 0, st>>>(
        n, nrhs, Nn, reinterpret_cast<const double2 *>(Zf), ldz, stride_z,
        reinterpret_cast<const double2 *>(band), mask_rows, reinterpret_cast<const double2 *>(X),
        reinterpret_cast<const double2 *>(B), ldb, stride_b, reinterpret_cast<double2 *>(R),
        reinterpret_cast<float2 *>(Rlo), norms);
    return check_launch("residual");
}

extern "C" int ghost_bor_residual_x32(int batch, int n, int nrhs, int Nn,
                                      const void *Zf, int z_split, long long ldz, long long stride_z,
                                      const double *band, const int *mask_rows,
                                      const float *X32, const double *B, long long ldb, long long stride_b,
                                      double *R, float *R32, double *norms, void *stream)
{
    if (batch < 1 || n < 1 || nrhs < 1 || !Zf || !mask_rows || !X32 || !B || (!R && !R32) || !norms ||
        ldz < n || ldb < nrhs || n != 2 * Nn)
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(norms, 0, sizeof(double) * 2 * batch, st) != cudaSuccess) return check_launch("residual_x32: memset");
    dim3 grid((nrhs + GT - 1) / GT, (n + GT - 1) / GT, batch);
    if (z_split)
        residual_mixed_kernel<float2, float4><<<grid, 256, 0, st>>>(
            n, nrhs, Nn, reinterpret_cast<const float4 *>(Zf), ldz, stride_z,
            reinterpret_cast<const double2 *>(band), mask_rows, reinterpret_cast<const float2 *>(X32),
            reinterpret_cast<const double2 *>(B), ldb, stride_b, reinterpret_cast<double2 *>(R),
            reinterpret_cast<float2 *>(R32), norms);
    else
        residual_mixed_kernel<float2, double2><<<grid, 256, 0, st>>>(
            n, nrhs, Nn, reinterpret_cast<const double2 *>(Zf), ldz, stride_z,
            reinterpret_cast<const double2 *>(band), mask_rows, reinterpret_cast<const float2 *>(X32),
            reinterpret_cast<const double2 *>(B), ldb, stride_b, reinterpret_cast<double2 *>(R),
            reinterpret_cast<float2 *>(R32), norms);
    return check_launch("residual_x32");
}

// in-place split of complex double into FP32 words (hi.re, hi.im, lo.re, lo.im)
__global__ void split_words_kernel(int rows, int cols, double2 *__restrict__ Z, long long ldz, long long sz)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    double2 *p = Z + (size_t)blockIdx.z * sz + (size_t)blockIdx.y * ldz + c;
    const float4 w = split_words(*p);
    *reinterpret_cast<float4 *>(p) = w;
}

extern "C" int ghost_bor_split_words(int batch, int rows, int cols, void *Z, long long ldz, long long stride_z,
                                     void *stream)
{
    if (batch < 1 || rows < 1 || cols < 1 || !Z || ldz < cols) return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    dim3 grid((cols + 255) / 256, rows, batch);
    split_words_kernel<<<grid, 256, 0, st>>>(rows, cols, reinterpret_cast<double2 *>(Z), ldz, stride_z);
    return check_launch("split_words");
}

extern "C" int ghost_bor_residual64(int batch, int n, int nrhs,
                                    const double *Z, long long ldz, long long stride_z,
                                    const double *X, const double *B, long long ldb, long long stride_b,
                                    double *R, double *norms, void *stream)
{
    if (batch < 1 || n < 1 || nrhs < 1 || !Z || !X || !B || !norms || ldz < n || ldb < nrhs)
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(norms, 0, sizeof(double) * 2 * batch, st) != cudaSuccess) return check_launch("residual64: memset");
    dim3 grid((nrhs + GT - 1) / GT, (n + GT - 1) / GT, batch);
    residual64_kernel<<<grid, 256, 0, st>>>(n, nrhs, reinterpret_cast<const double2 *>(Z), ldz, stride_z,
                                            reinterpret_cast<const double2 *>(X), reinterpret_cast<const double2 *>(B),
                                            ldb, stride_b, reinterpret_cast<double2 *>(R), norms);
    return check_launch("residual64");
}

extern "C" int ghost_bor_compose(int batch, int n, int Nn, const void *Zf, long long ldz, long long stride_z,
                                 const double *band, const int *mask_rows,
                                 void *A, long long lda, long long stride_a, void *stream)
{
    if (batch < 1 || n < 1 || n != 2 * Nn || !Zf || !mask_rows || !A || ldz < n || lda < n) return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    dim3 grid((n + 255) / 256, n, batch);
    compose_kernel<<<grid, 256, 0, st>>>(n, Nn, reinterpret_cast<const double2 *>(Zf), ldz, stride_z,
                                         reinterpret_cast<const double2 *>(band), mask_rows,
                                         reinterpret_cast<float2 *>(A), lda, stride_a);
    return check_launch("compose");
}

extern "C" int ghost_bor_mask64(int batch, int n, const int *mask_rows, double *Z, long long ldz, long long stride_z,
                                void *stream)
{
    if (batch < 1 || n < 1 || !mask_rows || !Z || ldz < n) return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    dim3 grid((n + 255) / 256, 4, batch);
    mask64_kernel<<<grid, 256, 0, st>>>(n, mask_rows, reinterpret_cast<double2 *>(Z), ldz, stride_z);
    return check_launch("mask64");
}

extern "C" int ghost_bor_convert(int dir, int batch, int rows, int cols,
                                 const void *src, long long lds, long long stride_s,
                                 void *dst, long long ldd, long long stride_d, void *stream)
{
    if (dir < 0 || dir > 3 || batch < 1 || rows < 1 || cols < 1 || !src || !dst || lds < cols || ldd < cols)
        return GHOST_BOR_EINVAL;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    dim3 grid((cols + 255) / 256, rows, batch);
    convert_kernel<<<grid, 256, 0, st>>>(dir, rows, cols, src, lds, stride_s, dst, ldd, stride_d);
    return check_launch("convert");
}
