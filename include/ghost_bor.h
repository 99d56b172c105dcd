/*
 * ghost_bor.h -- C ABI of the GB300 (sm_103a) body-of-revolution MoM path.
 *
 * Every function takes DEVICE pointers (caller-owned, allocated by the caller),
 * explicit sizes, and a CUDA stream passed as `void *` (NULL = legacy default
 * stream).  Kernels are launched asynchronously on that stream; the return
 * value only reports argument and launch errors.  Device-side numerical status
 * (zero pivots, iteration limits) is written to caller buffers named `info`.
 *
 * Complex arrays are interleaved (re, im) pairs of float (precision
 * GHOST_BOR_F32) or double (GHOST_BOR_F64).  Matrices are row-major with an
 * explicit leading dimension (elements between rows); batches of matrices are
 * separated by an explicit batch stride (elements).
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   sample_g / sample_mfie  bor_stream_kernel.c:26-48, 65-106 (ctypes binding
 *                           bor_streaming.py:50-73)
 *   far fill                bor_streaming.py:220-268 + 352-407
 *                           (StreamingFarBlocks._build_range, efie_blocks,
 *                           bracket_blocks)
 *   near fill               bor_solver.py:270-336 + bor_kernels.py:170-257
 *                           (_near_pair_data, modal_kernels_near, near loop of
 *                           assemble_mode); MFIE: bor_solver.py:372-435,
 *                           bor_kernels.py:334-431
 *   excitation              bor_solver.py:437-461, 625-645 (rhs_mfie_mode,
 *                           rhs_mode) for all modes x angles x polarisations
 *   LU + solves             bor_solver.py:753 (np.linalg.solve = zgesv)
 *   far field + mode sum    bor_solver.py:659-708, 771-801 (farfield_mode,
 *                           _mode_sweep accumulation)
 */
#ifndef GHOST_BOR_H
#define GHOST_BOR_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define GHOST_BOR_OK            0
#define GHOST_BOR_EINVAL        1   /* bad argument (size, pointer, alignment) */
#define GHOST_BOR_ECUDA         2   /* kernel launch / CUDA runtime error */
#define GHOST_BOR_EUNSUPPORTED  3   /* valid but unsupported configuration */

/* precisions */
#define GHOST_BOR_F32 0
#define GHOST_BOR_F64 1

/* Library version (major*10000 + minor*100 + patch). */
int ghost_bor_version(void);

/* Human-readable text of the last CUDA error seen by this library (thread-local). */
const char *ghost_bor_last_error(void);

/* Number of kernels this library has launched since it was loaded. */
long long ghost_bor_launch_count(void);

/* ------------------------------------------------------------------------
 * Drop-in device samplers.  Same argument meaning and output layout as the
 * reference ctypes functions, with device pointers and a stream:
 *   out[i][j][l] (interleaved complex double), i < nr, j < np_, l < nxi.
 * Replaces sample_g (bor_stream_kernel.c:26-48).
 */
int ghost_bor_sample_g(int nr, int np_, int nxi,
                       const double *rho_p, const double *z_p,
                       const double *rho_q, const double *z_q,
                       double k, const double *sin2_tab, double *out,
                       void *stream);

/* Replaces sample_mfie (bor_stream_kernel.c:65-106). */
int ghost_bor_sample_mfie(int nr, int np_, int nxi,
                          const double *rho_p, const double *z_p,
                          const double *tr_p, const double *tz_p,
                          const double *rho_q, const double *z_q,
                          const double *tr_q, const double *tz_q,
                          double k, const double *cos_tab, const double *sin_tab,
                          double *o_tt, double *o_tf, double *o_ft, double *o_ff,
                          void *stream);

/* Replaces sample_ibc (bor_stream_kernel.c:108-150): the four rotated
 * principal-value (IBC) brackets p(R) [(W_u . n')(R . f_v) - (W_u . f_v)(R . n')]
 * with the source normal n', same arguments and layout as ghost_bor_sample_mfie. */
int ghost_bor_sample_ibc(int nr, int np_, int nxi,
                         const double *rho_p, const double *z_p,
                         const double *tr_p, const double *tz_p,
                         const double *rho_q, const double *z_q,
                         const double *tr_q, const double *tz_q,
                         double k, const double *cos_tab, const double *sin_tab,
                         double *o_tt, double *o_tf, double *o_ft, double *o_ff,
                         void *stream);

/* ------------------------------------------------------------------------
 * Fused EFIE far fill: for every far element pair (|e - f| >= 2) sample the
 * Green's function on the half azimuth grid xi_j = pi j / (nxi/2), take the
 * even DCT to orders 0..m_max+1, contract with the Galerkin weights and
 * combine the orders into the mode-m blocks, m = 0..m_max, then ADD
 * scale * [[ztt, ztf], [zft, zff]] into Z[m] (rows 0..Nn-1 = J_t tests,
 * Nn..2Nn-1 = J_phi tests).  Z must be zeroed (or hold other terms) first.
 * `prec` selects the precision: GHOST_BOR_F64 = FP64 throughout;
 * GHOST_BOR_F32 = FP32 sampling (double-float phase) and DCT (Kahan-compensated
 * blocks), double-float contraction and mode combination, each entry rounded
 * to FP64 once before it is added.  Z is always complex double.
 *
 *   geo   [11][P] doubles, P = 4 n_elem (Gauss points, element-major):
 *         rho, z, w, T0*w*rho, T1*w*rho, T0*w, T1*w, dRT0*w, dRT1*w, t_rho, t_z
 *   dct   [nxi/2+1][m_max+2]  (pi/h) * c_j * cos(pi n j / h) / (4 pi),
 *                             c_0 = c_h = 1, else 2 (the kernel samples exp(-jkR)/R)
 *   sin2  [nxi/2+1]           sin^2(pi j / nxi)
 *   Z     complex double, Z[m] at Z + m*mode_stride, row stride ldz
 * Replaces StreamingFarBlocks._build_range + efie_blocks
 * (bor_streaming.py:220-268, 320-376, 388-407).
 */
int ghost_bor_far_efie(int prec, int n_elem, int m_max, int nxi, double k,
                       double scale_re, double scale_im,
                       const double *geo, const double *dct, const double *sin2,
                       void *Z, long long ldz, long long mode_stride,
                       void *stream);

/* ghost_bor_far_efie restricted to the far pairs (e, f) with elem_mask[e] or
 * elem_mask[f] nonzero (elem_mask: n_elem bytes on the device; NULL = all
 * pairs; used by the adjoint gradient to fill the operator change of a local
 * shape perturbation), and optionally reading the FP32 path's DCT table from
 * dct32 (fl32 of `dct`, same layout; NULL = convert `dct` on the fly).  No
 * counterpart in the reference. */
int ghost_bor_far_efie_masked(int prec, int n_elem, int m_max, int nxi, double k,
                              double scale_re, double scale_im,
                              const double *geo, const double *dct, const double *sin2,
                              void *Z, long long ldz, long long mode_stride,
                              const unsigned char *elem_mask, const float *dct32, void *stream);

/* Tensor-core form of the FP32-pipe EFIE far fill: the same contraction, mode
 * combination and accumulation as ghost_bor_far_efie(GHOST_BOR_F32, ...), with
 * (i) Green's-function samples as pairs of FP32 words accurate to ~3e-9 (a
 * double-float phase and table-driven sin / cos instead of sincosf), (ii) the
 * even DCT over the azimuth samples on the bf16 tensor cores (tcgen05) from
 * four balanced 8-bit integer digits of the samples and of the table, one
 * TMEM accumulator per digit level, and (iii) each far element pair sampled
 * once and contracted in both orientations (the kernel is symmetric in the
 * point pair).  The operator agrees with the FP64 fill to ~4e-9 of its largest
 * entry (the SIMT FP32 fill: ~7e-8).  Z is complex double; the contribution
 * is ADDED.
 *   work  ghost_bor_far_efie_tc_workspace(n_elem, m_max, nxi) bytes,
 *         256-byte aligned, prepared once per (m_max, nxi, table) by
 *         ghost_bor_far_efie_tc_tables from the `dct` / `sin2` tables of
 *         ghost_bor_far_efie (any n_elem's workspace holds the tables; the
 *         rest is room for the geometry rows as double-float words, which
 *         each fill call writes from `geo` before its transform); its first
 *         int is a status word, set to 1 if a bounded pipeline wait gave up
 *         (the launch is then incomplete).
 * Returns GHOST_BOR_EUNSUPPORTED when nxi/2 + 1 exceeds 2^17 samples.
 * Replaces StreamingFarBlocks._build_range + efie_blocks
 * (bor_streaming.py:220-268, 320-376, 388-407) like ghost_bor_far_efie. */
long long ghost_bor_far_efie_tc_workspace(int n_elem, int m_max, int nxi);
int ghost_bor_far_efie_tc_tables(int m_max, int nxi, const double *dct, const double *sin2,
                                 void *work, long long work_bytes, void *stream);
int ghost_bor_far_efie_tc(int n_elem, int m_max, int nxi, double k,
                          double scale_re, double scale_im, const double *geo,
                          void *work, long long work_bytes,
                          void *Z, long long ldz, long long mode_stride, void *stream);

/* ghost_bor_far_efie_tc restricted to the far pairs (e, f) with elem_mask[e]
 * or elem_mask[f] nonzero (n_elem bytes on the device; NULL = all pairs): the
 * tiles without such a pair are skipped.  Used by the adjoint gradient for the
 * operator change of a local shape perturbation.  No counterpart in the
 * reference. */
int ghost_bor_far_efie_tc_masked(int n_elem, int m_max, int nxi, double k,
                                 double scale_re, double scale_im, const double *geo,
                                 const unsigned char *elem_mask, void *work, long long work_bytes,
                                 void *Z, long long ldz, long long mode_stride, void *stream);

/* Persistent grid of the near fills: CTAs per SM (default: 2 for the
 * per-thread kernels, every resident CTA for the grouped double-float EFIE
 * kernel; 0 restores the defaults, at most 8).  The workspace size
 * (ghost_bor_near_workspace, ghost_bor_near_mfie_workspace) depends on it:
 * query it after a change.  A tuning knob, process-wide.  No counterpart in
 * the reference. */
int ghost_bor_set_near_grid(int ctas_per_sm);

/* ------------------------------------------------------------------------
 * FP64-class near/self EFIE fill for the element pairs (e, f), |e - f| <= 1, with
 * the graded-cell + sinh-core + Gauss-tail quadrature of the reference.
 *   nodes     [Nn][2] (rho, z);  elem [3][n_elem] (length, t_rho, t_z)
 *   pairs     [n_pairs][4] ints: e, f, cell-table offset, cell count
 *   tails     [n_pairs][2] ints: tail-table offset, n_tail
 *   cells     [3][n_cells_total] (s, s', w)
 *   core_gl   [2][48] (u01, w01);  tail_gl [4][n_tail_total] (u01, w01,
 *             sin and cos of xi/2 at the node for the core bound s0 = 1/4,
 *             xi = xi0 + u01 (pi - xi0), xi0 = 2 asin(1/4))
 * Output: if band != NULL, ADD scale * block into band[m][blk][Nn][5]
 * (complex double, blk = tt, tf, ft, ff; column offset -2..2); else into the
 * dense complex double Z[m].  `prec` selects the arithmetic: GHOST_BOR_F64 =
 * FP64 throughout; GHOST_BOR_F32 = double-float (two FP32 words, ~48-bit) on
 * the FP32 pipe for the azimuth-node transcendentals, the cos(m xi) projection
 * and the order GEMM (agrees with the FP64 result to ~3e-11 of each mode's
 * largest band entry).  For m_max + 2 <= 256 the F32 fill runs a grouped
 * kernel: 2..16 lanes share a point pair, each holding every G-th order in
 * registers, so the azimuth nodes never leave the chip; otherwise (and for
 * F64) each CTA of the persistent grid keeps the nodes of its 128 point pairs
 * in the workspace, so the transcendental functions still run once per node.
 * work: ghost_bor_near_workspace(n_tail_max) bytes, 256-byte aligned, where
 * n_tail_max >= every n_tail of `tails`; its first int is a status word set to
 * 1 if a pair had a larger n_tail (that pair is then skipped); it also holds
 * the double-float tail rule of each CTA's current pair.
 * Replaces _near_pair_data + modal_kernels_near + the near loop of
 * assemble_mode (bor_solver.py:270-336, bor_kernels.py:170-257).
 */
long long ghost_bor_near_workspace(int n_tail_max);
int ghost_bor_near_efie(int prec, int n_elem, int m_max, double k,
                        double scale_re, double scale_im,
                        const double *nodes, const double *elem,
                        int n_pairs, const int *pairs, const int *tails,
                        const double *cells, int n_cells_total,
                        const double *core_gl, const double *tail_gl, int n_tail_total,
                        double *band, void *Z, long long ldz, long long mode_stride,
                        int n_tail_max, void *work, long long work_bytes, void *stream);

/* ------------------------------------------------------------------------
 * Fused MFIE far fill: for every far element pair (|e - f| >= 2) sample
 * p(R) = (1 + j k R) e^{-j k R} / R^3 on the half bracket grid
 * xi_j = pi j / (nxi/2), take the three transforms in `tab`, form the four
 * bracket blocks K_tt, K_tf, K_ft, K_ff of the reference (exact
 * rearrangement: every bracket is p (u + v s2) or sin(xi) p (u + v s2) with
 * per-point-pair constants), contract with the weights T w rho on both sides
 * and ADD -scale * [[K_tt, K_tf], [K_ft, K_ff]] into Z[m], m = 0..m_max
 * (the far part of Z_MFIE = M/2 - K; K(-m) = D K(m) D with D = diag(I, -I)).
 * `prec` selects the sampling / transform arithmetic; the contraction and
 * the accumulation into Z are FP64.
 *   geo   as in ghost_bor_far_efie
 *   tab   [3][nxi/2+1][m_max+1]: (pi/nxi) c_j cos(m xi_j),
 *         (pi/nxi) c_j sin^2(xi_j/2) cos(m xi_j), (pi/nxi) 2 sin(xi_j) sin(m xi_j)
 *   sin2  [nxi/2+1] sin^2(xi_j / 2);  nxi = the bracket rule
 *         (bor_streaming.py:114-116)
 * Replaces sample_mfie + the bracket FFT and contraction of
 * StreamingFarBlocks (bor_stream_kernel.c:65-106, bor_streaming.py:241-246,
 * 378-385, 409-421).
 */
int ghost_bor_far_mfie(int prec, int n_elem, int m_max, int nxi, double k,
                       double scale_re, double scale_im,
                       const double *geo, const double *tab, const double *sin2,
                       void *Z, long long ldz, long long mode_stride, void *stream);

/* ------------------------------------------------------------------------
 * FP64 near MFIE blocks (|e - f| <= 1) on the graded cells of
 * ghost_bor_near_efie, with the bracket grid of the reference (sinh core
 * with s0 = 1 for on-axis points + Gauss tail, +xi and -xi folded), plus the
 * mass term: ADD scale * (M/2 - K) for m = 0..m_max into the band or the
 * dense Z (layouts as in ghost_bor_near_efie).
 *   emass [n_elem][4] element mass contributions 2 pi sum_g T_a T_b w rho
 *         for (a, b) = (0,0), (0,1), (1,0), (1,1)
 *   work  ghost_bor_near_mfie_workspace(n_tail_max) bytes, as in
 *         ghost_bor_near_efie
 * Replaces mfie_kernels_near, _near_mfie_data, mass_blocks and the near loop
 * of assemble_mfie_mode (bor_kernels.py:334-431, bor_solver.py:372-435).
 */
long long ghost_bor_near_mfie_workspace(int n_tail_max);
int ghost_bor_near_mfie(int n_elem, int m_max, double k, double scale_re, double scale_im,
                        const double *nodes, const double *elem, const double *emass,
                        int n_pairs, const int *pairs, const int *tails,
                        const double *cells, int n_cells_total,
                        const double *core_gl, const double *tail_gl, int n_tail_total,
                        double *band, void *Z, long long ldz, long long mode_stride,
                        int n_tail_max, void *work, long long work_bytes, void *stream);

/* ------------------------------------------------------------------------
 * Surface-impedance (IBC-EFIE) operator addition Z_s (M/2) + B for
 * m = 0..m_max: the Z_s-weighted mass term plus the rotated principal-value
 * brackets B_uv = p(R) W_u . [R x (n' x f_v)] with Z_s at the source.  Both
 * fills ADD scale * Z_s(f) * (block) for every pair (e, f), Z_s(f) the complex
 * impedance of the source element:
 *   zs_elem [n_elem] complex (interleaved re, im), or NULL for Z_s = 1
 * ghost_bor_far_ibc: the far pairs |e - f| >= 2, arguments otherwise as in
 *   ghost_bor_far_mfie (same tables, same bracket rule for nxi).
 *   Replaces sample_ibc + the streamed IBC blocks and _rot_pv_blocks' far
 *   part (bor_stream_kernel.c:108-150, bor_kernels.py:449-511,
 *   bor_solver.py:499-519).
 * ghost_bor_near_ibc: the near pairs |e - f| <= 1 on the graded cells and the
 *   mass term (self pairs), arguments otherwise as in ghost_bor_near_mfie
 *   (workspace ghost_bor_near_mfie_workspace).  Replaces ibc_kernels_near,
 *   _near_ibc_data, the near loop of _rot_pv_blocks and mass_blocks(weight)
 *   (bor_kernels.py:514-560, bor_solver.py:481-497, 520-552).
 */
int ghost_bor_far_ibc(int prec, int n_elem, int m_max, int nxi, double k,
                      double scale_re, double scale_im, const double *zs_elem,
                      const double *geo, const double *tab, const double *sin2,
                      void *Z, long long ldz, long long mode_stride, void *stream);
int ghost_bor_near_ibc(int n_elem, int m_max, double k, double scale_re, double scale_im,
                       const double *zs_elem, const double *nodes, const double *elem,
                       const double *emass, int n_pairs, const int *pairs, const int *tails,
                       const double *cells, int n_cells_total,
                       const double *core_gl, const double *tail_gl, int n_tail_total,
                       double *band, void *Z, long long ldz, long long mode_stride,
                       int n_tail_max, void *work, long long work_bytes, void *stream);

/* ------------------------------------------------------------------------
 * FP64 fills with a complex wave number k = k_re + j k_im, k_im <= 0 (the
 * interior of a lossy medium, for the PMCHWT operators T_i and P_i;
 * bor_solver.py:161-200): the samples gain e^{k_im R}, p(R) becomes
 * (1 - k_im R + j k_re R) e^{k_im R} (cos - j sin) / R^3 and 1/k^2 is complex.
 * Arguments as in ghost_bor_far_efie (FP64, no element mask),
 * ghost_bor_near_efie (FP64 path), ghost_bor_far_ibc and ghost_bor_near_ibc;
 * nxi, the cells and the tail orders come from |k| as the reference forms
 * them for a complex k.
 */
int ghost_bor_far_efie_ck(int n_elem, int m_max, int nxi, double k_re, double k_im,
                          double scale_re, double scale_im,
                          const double *geo, const double *dct, const double *sin2,
                          void *Z, long long ldz, long long mode_stride, void *stream);
int ghost_bor_near_efie_ck(int n_elem, int m_max, double k_re, double k_im,
                           double scale_re, double scale_im,
                           const double *nodes, const double *elem,
                           int n_pairs, const int *pairs, const int *tails,
                           const double *cells, int n_cells_total,
                           const double *core_gl, const double *tail_gl, int n_tail_total,
                           double *band, void *Z, long long ldz, long long mode_stride,
                           int n_tail_max, void *work, long long work_bytes, void *stream);
int ghost_bor_far_ibc_ck(int n_elem, int m_max, int nxi, double k_re, double k_im,
                         double scale_re, double scale_im, const double *zs_elem,
                         const double *geo, const double *tab, const double *sin2,
                         void *Z, long long ldz, long long mode_stride, void *stream);
int ghost_bor_near_ibc_ck(int n_elem, int m_max, double k_re, double k_im,
                          double scale_re, double scale_im, const double *zs_elem,
                          const double *nodes, const double *elem, const double *emass,
                          int n_pairs, const int *pairs, const int *tails,
                          const double *cells, int n_cells_total,
                          const double *core_gl, const double *tail_gl, int n_tail_total,
                          double *band, void *Z, long long ldz, long long mode_stride,
                          int n_tail_max, void *work, long long work_bytes, void *stream);

/* ------------------------------------------------------------------------
 * Excitation for all modes 0..m_max, angles and both polarisations:
 *   B[m][row][2*it + pol] (complex double, row stride ldb, mode stride),
 *   pol 0 = VV (theta), 1 = HH (phi).  Rows flagged in mask_rows[m][4]
 *   (-1 = unused) are written as zero.
 *   coef_e multiplies the EFIE excitation <W, E_inc> (rhs_mode),
 *   coef_h multiplies the rotated MFIE excitation <W, n x H_inc>
 *   (rhs_mfie_mode); either may be 0.
 *   geo as in ghost_bor_far_efie; thetas_deg [n_theta].
 *   work: caller scratch of ghost_bor_rhs_workspace() bytes.
 * Bessel J_n by Miller's backward recurrence (FP64).
 */
long long ghost_bor_rhs_workspace(int n_elem, int m_max, int n_theta);
int ghost_bor_rhs(int n_elem, int m_max, int n_theta, double k,
                  double coef_e, double coef_h,
                  const double *geo, const double *thetas_deg,
                  const int *mask_rows, double *B, long long ldb, long long mode_stride,
                  void *work, void *stream);

/* ghost_bor_rhs with a complex weight per element on the n x H part:
 * coef_e <W, E_inc> + coef_h <W, h_weight(el) n x H_inc>, h_weight
 * [n_elem] complex (interleaved re, im, not NULL).  With coef_e = 1,
 * coef_h = -1 and h_weight = Z_s this is the reciprocity vector of the far
 * field of an impedance surface, J plus the eliminated M = -Z_s n x J
 * (farfield_mode with zs_pt, bor_solver.py:659-708).
 */
int ghost_bor_rhs_weighted(int n_elem, int m_max, int n_theta, double k,
                           double coef_e, double coef_h, const double *h_weight,
                           const double *geo, const double *thetas_deg,
                           const int *mask_rows, double *B, long long ldb, long long mode_stride,
                           void *work, void *stream);

/* Allocation-free variant of ghost_bor_rhs for callers that cannot allocate
 * device memory during a solve (a service that reserves all GPU memory up front,
 * or a thread that must not call cudaMalloc/cudaFree because they can
 * synchronise the device).  Same arguments and output as ghost_bor_rhs minus
 * `work`: the workspace is a 64 MiB static device array owned by the library
 * (held on every GPU that loads it until exit), used in blocks of angles.
 * Rejects (GHOST_BOR_EINVAL) problems where one angle needs more than the
 * array: 4*n_elem*((m_max+2)*8 + 16) > 64 MiB - 256.  Calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller.  The
 * first call on a device looks the array up (cudaGetSymbolAddress) and should
 * come before any stream capture; the looked-up address is kept for the life
 * of the process, so it is stale after cudaDeviceReset of that device (do not
 * call this entry point on a device after resetting it).  No counterpart in
 * the reference.
 * ghost_bor_rhs_noalloc_capacity() returns the array size in bytes. */
long long ghost_bor_rhs_noalloc_capacity(void);
int ghost_bor_rhs_noalloc(int n_elem, int m_max, int n_theta, double k,
                          double coef_e, double coef_h,
                          const double *geo, const double *thetas_deg,
                          const int *mask_rows, double *B, long long ldb, long long mode_stride,
                          void *stream);

/* ------------------------------------------------------------------------
 * Batched complex LU with partial pivoting (|re|+|im| pivot rule, as LAPACK
 * izamax) of n x n matrices A[b] = A + b*stride_a, row-major, b < batch.
 * ipiv[b][n] receives 0-based pivot rows; info[b] = 0 or (first zero pivot
 * column + 1).  In place.  For GHOST_BOR_F32 with a workspace of
 * ghost_bor_getrf_workspace() bytes (256-byte aligned) the trailing updates
 * run on the tensor cores (ghost_bor_cgemm_tc); the first int of the
 * workspace is then a sticky status (1 = a bounded in-kernel wait gave up).
 * work = NULL selects the SIMT updates (always for FP64).
 */
long long ghost_bor_getrf_workspace(int prec, int batch, int n);
int ghost_bor_getrf(int prec, int batch, int n, void *A, long long lda, long long stride_a,
                    int *ipiv, int *info, void *work, void *stream);

/* Complex FP32 update C[b] -= A[b] B[b] on the tensor cores (tcgen05
 * kind::tf32, 3xTF32 split, TMA-staged operands, TMEM accumulator):
 * A [M][K], B [K][N], C [M][N] row-major complex float with leading
 * dimensions lda/ldb/ldc and batch strides (complex elements).
 * work: ghost_bor_cgemm_tc_workspace() bytes of device scratch.  status
 * (device int, may be NULL) receives 1 if a bounded in-kernel wait gave up.
 * Building block of the LU trailing updates and the triangular solves. */
long long ghost_bor_cgemm_tc_workspace(int batch, int M, int N, int K);
/* Polls of each pipeline wait (mbarrier) in the GEMM update kernel before it
 * gives up, sets its status word and returns (default 2^24; polls < 0 restores
 * it; 0 makes the first wait give up at once).  The kernel still waits, with
 * the default limit, for its copies and MMAs in flight before it exits.  A
 * test hook for the error path of the bounded waits; process-wide, not thread
 * safe against concurrent launches.  No counterpart in the reference. */
void ghost_bor_set_wait_limit(long long polls);
int ghost_bor_cgemm_tc(int batch, int M, int N, int K,
                       const void *A, long long lda, long long stride_a,
                       const void *B, long long ldb, long long stride_b,
                       void *C, long long ldc, long long stride_c,
                       void *work, int *status, void *stream);

/* Solve A X = B with the factors of ghost_bor_getrf for nrhs columns
 * (B row-major n x nrhs, in place).  Precisions of A and B are equal; work as
 * for ghost_bor_getrf (ghost_bor_getrs_workspace() bytes, or NULL). */
long long ghost_bor_getrs_workspace(int prec, int batch, int n, int nrhs);
int ghost_bor_getrs(int prec, int batch, int n, int nrhs,
                    const void *A, long long lda, long long stride_a, const int *ipiv,
                    void *B, long long ldb, long long stride_b, void *work, void *stream);

/* ------------------------------------------------------------------------
 * Mixed-precision residual for iterative refinement, per batch b:
 *   R = B - (Zf + band) X        with Zf complex double (far part), band
 *   complex double [Nn blocks as in ghost_bor_near_efie] (may be NULL), X and
 *   B complex double; rows in mask_rows[b] produce R = 0.
 * If Rlo != NULL the residual is also written as complex float to Rlo.
 * norms[b][2] receives (||R||_F^2, ||B||_F^2).
 * Zf and X are split into two FP32 words each; the leading products are
 * summed in FP32 over 4-term chunks and across chunks in double-float.
 */
int ghost_bor_residual(int batch, int n, int nrhs, int Nn,
                       const void *Zf, long long ldz, long long stride_z,
                       const double *band, const int *mask_rows,
                       const double *X, const double *B, long long ldb, long long stride_b,
                       double *R, float *Rlo, double *norms, void *stream);

/* Residual of an FP32 solution X32 (complex float, same ldb / stride_b as B):
 *   R = B - (Zf + band) X32, with the arithmetic of ghost_bor_residual (the
 *   low FP32 word of X is zero, so the Z_hi X_lo products drop out).
 * R (complex double) and R32 (complex float) are each optional, not both.
 * z_split = 1: Zf holds the FP32 words (hi.re, hi.im, lo.re, lo.im) written by
 * ghost_bor_split_words instead of complex double (same 16 bytes per element),
 * which takes the FP64 splitting out of the tile staging.
 * The first residual of the refinement; later residuals follow from it by
 * R -= fl32(Z) D for each correction D (ghost_bor_cgemm_tc).  No counterpart in
 * the reference (its solve is FP64 LAPACK, bor_solver.py:753-756). */
int ghost_bor_residual_x32(int batch, int n, int nrhs, int Nn,
                           const void *Zf, int z_split, long long ldz, long long stride_z,
                           const double *band, const int *mask_rows,
                           const float *X32, const double *B, long long ldb, long long stride_b,
                           double *R, float *R32, double *norms, void *stream);

/* FP64 residual R = B - Z X (all complex double); norms as above. */
int ghost_bor_residual64(int batch, int n, int nrhs,
                         const double *Z, long long ldz, long long stride_z,
                         const double *X, const double *B, long long ldb, long long stride_b,
                         double *R, double *norms, void *stream);

/* ------------------------------------------------------------------------
 * Far field by reciprocity + mode weights:
 *   dF[b][c] = pref * wt[b] * sgn(c) * sum_i d_i Ve[b][i][c] X[b][i][c]
 * d_i = +1 for rows < Nn (J_t), -1 otherwise; sgn(c) = +1 for even c (VV),
 * -1 for odd c (HH); pref = -j k eta0 / (4 pi).  X precision prec; Ve double.
 * Replaces farfield_mode (bor_solver.py:659-708).
 */
int ghost_bor_farfield(int prec, int batch, int n, int nrhs, int Nn, double k,
                       const double *mode_weight,
                       const double *Ve, long long ldv, long long stride_v,
                       const void *X, long long ldx, long long stride_x,
                       double *dF, void *stream);

/* ------------------------------------------------------------------------
 * Small helpers used between stages.
 * ghost_bor_compose: A32[b] = fl32(Zf[b] + band[b]) (Zf complex double, A32
 *   complex float) with masked rows/columns replaced by identity rows/columns
 *   (band may be NULL).
 * ghost_bor_mask64: apply the same identity masking to a complex double Z.
 * ghost_bor_convert: elementwise complex copy of a strided batch of row
 *   blocks (dir 0: double->float, 1: float->double, 2: float added into
 *   double, 3: float->float).
 */
/* Refinement residual with exact products on the bf16 tensor cores (Ozaki
 * splitting): R = B - (Zf + band) X32 with Zf complex double, X32 the FP32
 * solution (same ldb / stride_b as B).  Rows of Zf and columns of X32 are
 * scaled by powers of two and split into four 8-bit integer slices (exact in
 * bf16); slice products are accumulated exactly in FP32 TMEM over K chunks of
 * 192 and folded into double-float accumulators, so the residual carries
 * ~2^-31 of the row / column scales instead of the ~2^-24 of FP32 products.
 * R and R32 optional (not both NULL); norms as in ghost_bor_residual, summed
 * in FP32 per thread (relative accuracy ~1e-7, enough for a stopping test).
 * work: ghost_bor_residual_exact_workspace(batch, n, nrhs) bytes, 256-byte
 * aligned; its first int is set to 1 if a bounded in-kernel wait gave up.
 * No counterpart in the reference (its solve is FP64 LAPACK). */
long long ghost_bor_residual_exact_workspace(int batch, int n, int nrhs);
int ghost_bor_residual_exact(int batch, int n, int nrhs, int Nn,
                             const double *Zf, long long ldz, long long stride_z,
                             const double *band, const int *mask_rows,
                             const float *X32, const double *B, long long ldb, long long stride_b,
                             double *R, float *R32, double *norms,
                             void *work, long long work_bytes, void *stream);

/* In place: complex double Z -> its two FP32 words (hi.re, hi.im, lo.re, lo.im),
 * hi = fl32(z), lo = fl32(z - hi). */
int ghost_bor_split_words(int batch, int rows, int cols, void *Z, long long ldz, long long stride_z,
                          void *stream);
int ghost_bor_compose(int batch, int n, int Nn, const void *Zf, long long ldz, long long stride_z,
                      const double *band, const int *mask_rows,
                      void *A, long long lda, long long stride_a, void *stream);
int ghost_bor_mask64(int batch, int n, const int *mask_rows,
                     double *Z, long long ldz, long long stride_z, void *stream);
int ghost_bor_convert(int dir, int batch, int rows, int cols,
                      const void *src, long long lds, long long stride_s,
                      void *dst, long long ldd, long long stride_d, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GHOST_BOR_H */
