/*
 * nt_gb300.h -- C ABI of the GB300 (sm_103a) kernels behind the analytic
 * NNGP/NTK path of neural-tangents (nt.stax kernel_fn, nt.batch,
 * nt.predict.gradient_descent_mse).
 *
 * Conventions
 *   - Every entry point returns 0 on success or a positive NTG_ERR_* code;
 *     ntg_last_error() returns a message for the calling thread.
 *   - `stream` is a cudaStream_t passed as void* (0 = legacy default stream).
 *   - All buffers are device pointers to contiguous float32 arrays unless a
 *     comment says float64; the caller owns every buffer. Work is enqueued
 *     on `stream`; no entry point synchronises unless its comment says so.
 *   - Kernel tensors use the reference's zipped layout: a pair tensor
 *     (nngp, ntk) is [B, A, A', C, C'] with B = N1*N2 pairs in row-major
 *     (n1, n2) order; a per-sample tensor (cov1, cov2) is [N, A, A', C, C'].
 *     One spatial dimension is passed as C = 1; no spatial dimension
 *     (fully-connected kernels) as A = C = 1.
 *   - A "variance" operand is the diagonal of a pre-activation per-sample
 *     kernel, addressed as base + n*s_n + a*s_a + c*s_c.
 */
#ifndef NT_GB300_H_
#define NT_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  NTG_OK = 0,
  NTG_ERR_INVALID_ARG = 1,
  NTG_ERR_CUDA = 2,
  NTG_ERR_UNSUPPORTED = 3,
  NTG_ERR_NOT_POSITIVE_DEFINITE = 4,
  NTG_ERR_WAIT_TIMEOUT = 5,
  NTG_ERR_NO_DEVICE_SCRATCH = 6
};

enum {
  NTG_ACT_NONE = 0,
  NTG_ACT_ABRELU = 1,
  NTG_ACT_ERF = 2,
  NTG_ACT_SIN = 3,  /* a sin(b x + c) (Cos: c + pi/2), elementwise.py:275-345; the `c`
                       field of ntg_act_t carries cos(2 c) */
  NTG_ACT_RBF = 4,  /* gamma in `a`, elementwise.py:348-400 */
  NTG_ACT_GELU = 5  /* elementwise.py:195-272 */
};
enum { NTG_PAD_ZERO = 0, NTG_PAD_CIRCULAR = 1 };

/* Activation rule applied to (nngp, ntk) given var1 (first sample) and var2
 * (second sample).  ABRelu(a, b): neural_tangents/_src/stax/elementwise.py:403-477
 * (Relu = ABRelu(0, 1)).  Erf(a, b, c): elementwise.py:47-114.
 * `compensated` = 1 evaluates var1*var2 - q^2 as an exact two-product
 * difference (accurate near correlation +-1); 0 follows the plain float32
 * formula of the reference. `stabilize` > 0 is the do_stabilize factor
 * (ABRelu only; elementwise.py:431-436, 462-466). */
typedef struct {
  int32_t kind;
  float a, b, c;
  int32_t compensated;
  float stabilize;
} ntg_act_t;

/* Affine rule of Dense / Conv on an (unscaled) propagated kernel u:
 *   nngp_out = w2 * u + b2
 *   ntk_out  = ntk_w2 * u_ntk + ntk_nn * (nn_scaled ? nngp_out : u) + ntk_c
 * NTK parameterisation: ntk_w2 = W^2, ntk_nn = 1, nn_scaled = 1, ntk_c = 0
 * (neural_tangents/_src/stax/linear.py:906-911, 1394-1398); standard:
 * ntk_nn = fan_in / s0, nn_scaled = 0, ntk_c = (b_std given) (linear.py:912-919,
 * 1400-1406). */
typedef struct {
  float w2, b2;
  float ntk_w2, ntk_nn, ntk_c;
  int32_t nn_scaled;
} ntg_affine_t;

/* Strided view of per-sample variances (diagonal of a per-sample kernel). */
typedef struct {
  const float* base;
  int64_t s_n, s_a, s_c;
} ntg_var_t;

/* ---- library ---------------------------------------------------------- */
const char* ntg_last_error(void);
const char* ntg_version(void);
/* Number of sm_103a kernels launched by this library since load (all threads). */
uint64_t ntg_launch_count(void);
/* Reads and clears the device error word of the streamed kernels (synchronous):
 * NTG_ERR_WAIT_TIMEOUT if a bounded pipeline wait ran out since the last call. */
int ntg_device_status(void);

/* ---- tuning (process-wide, thread-safe) --------------------------------- */
/* Launch parameters an autotuner may change (no counterpart in the reference,
 * where XLA chooses its own). Values are checked; results do not depend on them.
 *   NTG_TUNE_STENCIL_RING: input planes in flight per CTA of the 32 x 32
 *     full-spatial stencil of ntg_conv_fs — 2, 3, 4 (default) or 6. */
enum { NTG_TUNE_STENCIL_RING = 0, NTG_TUNE_COUNT = 1 };
int ntg_tune_set(int32_t knob, int32_t value);
/* Current value of a knob, or -1 for an unknown knob. */
int32_t ntg_tune_get(int32_t knob);

/* ---- input kernels (requirements.py:518-638, 641-830) ---------------- */
/* Flat inputs x1 [N1, D], x2 [N2, D] -> nngp [N1, N2] = x1 x2^T / D
 * (requirements.py:542-564). precision 0: FP32 on CUDA cores, every entry an
 * fmaf chain in ascending D (workspace unused, may be NULL); 1: x = hi + lo
 * split into BF16, hi1 hi2^T + hi1 lo2^T + lo1 hi2^T on the tcgen05 tensor
 * cores with FP32 accumulation, fed by TMA (a persistent kernel, one CTA per
 * SM); needs ntg_gram_workspace_bytes(n1, n2, d) bytes of workspace, whose
 * first int32 is set non-zero if a bounded pipeline wait ran out (read it
 * back, or ntg_device_status). When x1 == x2 (the same pointer) and n1 == n2
 * both precisions compute the tiles on or below the diagonal only and store
 * each also transposed: the output is exactly symmetric (for precision 0 bit
 * for bit what two distinct copies of x would give). */
int ntg_gram(void* stream, const float* x1, const float* x2, int64_t n1, int64_t n2,
             int64_t d, float* nngp, int32_t precision, void* workspace, size_t workspace_bytes);
size_t ntg_gram_workspace_bytes(int64_t n1, int64_t n2, int64_t d);
/* C [m, n] = A [m, k] B [k, n] in FP32 (C += A B when accumulate != 0): the
 * tensordot(k_test_train, solve(...)) of predict.py:172-174. */
int ntg_gemm(void* stream, const float* a, const float* b, float* c, int64_t m, int64_t n,
             int64_t k, int32_t accumulate);
/* Per-row sum(x^2)/D -> cov [N] (requirements.py:518-526, 572-582). */
int ntg_cov_diag(void* stream, const float* x, int64_t n, int64_t d, float* cov);
/* Image inputs x1 [N1, A, C, K], x2 [N2, A, C, K] (NHWC, K channels) ->
 * full-spatial nngp [N1, N2, A, A, C, C] = sum_k x1 x2 / K
 * (requirements.py:542-553). With x2 == x1 and pairs == 0 writes the
 * per-sample cov [N, A, A, C, C] (requirements.py:529-539). */
int ntg_input_fs(void* stream, const float* x1, const float* x2, int64_t n1, int64_t n2,
                 int64_t a, int64_t c, int64_t k, int32_t pairs, float* out);
/* Diagonal-spatial input covariances (requirements.py:641-830 with
 * diagonal_spatial = True): x1 [N1, P, K], x2 [N2, P, K] over P spatial
 * positions -> nngp [N1, N2, P] = sum_k x1 x2 / K; with x2 == NULL and n2 == 0
 * the per-sample cov [N1, P] (same channel order, so self pairs agree exactly). */
int ntg_input_ds(void* stream, const float* x1, const float* x2, int64_t n1, int64_t n2,
                 int64_t p, int64_t k, float* out);

/* ---- Conv / Dense / activations on materialised kernels --------------- */
/* Full-spatial shared-weight convolution rule (linear.py:1321-1424,
 * 3115-3207, 3341-3378) on a [B, A, A, C, C] kernel, fused with the affine
 * rule and an optional activation epilogue.  Filter (fh, fw), strides
 * (sh, sw), low padding (ph, pw); output spatial size (ao, co); pad_mode
 * NTG_PAD_ZERO (SAME/VALID) or NTG_PAD_CIRCULAR.  in_ntk may be NULL (the
 * scalar-zero NTK of an input kernel, or no NTK).  out_ntk may be NULL.
 * For act.kind != NONE, var1/var2 are the pre-activation variances of the
 * OUTPUT (diagonal of the convolved per-sample kernels) and n2 > 0 maps pair
 * b to samples (b / n2, b % n2); n2 == 0 means per-sample (b, b). */
int ntg_conv_fs(void* stream, const float* in_nngp, const float* in_ntk,
                float* out_nngp, float* out_ntk, int64_t batch, int64_t n2,
                int64_t a, int64_t c, int32_t fh, int32_t fw, int32_t sh, int32_t sw,
                int32_t ph, int32_t pw, int64_t ao, int64_t co, int32_t pad_mode,
                ntg_affine_t aff, ntg_act_t act, ntg_var_t var1, ntg_var_t var2);
/* First Conv fused with the input Gram: x1 [N1, A, C, K], x2 [N2, A, C, K]
 * -> conv(x1 x2^T / K) with affine + activation, written as [N1*N2, A, A, C, C]
 * (3x3 / stride 1 / SAME / zero padding). ntk_out = nngp_out before the
 * activation, as for an input kernel whose NTK is the scalar zero. */
/* ntg_conv_fs for a 3x3 / stride 1 / SAME / zero-padded conv on 32 x 32 planes
 * followed by an activation, also writing the conv output before the activation
 * (pre_q, pre_t) that the activation's VJP needs: one pass instead of a conv and
 * an activation pass. NTG_ERR_UNSUPPORTED for other shapes or unaligned buffers
 * (run ntg_conv_fs and ntg_affine_act then). No reference counterpart. */
int ntg_conv_act_fs(void* stream, const float* in_q, const float* in_t, float* out_q,
                    float* out_t, float* pre_q, float* pre_t, int64_t batch, int64_t n2,
                    int64_t a, int64_t c, ntg_affine_t aff, ntg_act_t act, ntg_var_t var1,
                    ntg_var_t var2);
int ntg_conv_input_fs(void* stream, const float* x1, const float* x2, int64_t n1, int64_t n2,
                      int64_t a, int64_t c, int64_t k, float* out_nngp, float* out_ntk,
                      ntg_affine_t aff, ntg_act_t act, ntg_var_t var1, ntg_var_t var2);
/* Diagonal-spatial convolution (linear.py:3381-3437): [B, A, C] box filter. */
int ntg_conv_ds(void* stream, const float* in_nngp, const float* in_ntk, float* out_nngp,
                float* out_ntk, int64_t batch, int64_t a, int64_t c, int32_t fh, int32_t fw,
                int32_t sh, int32_t sw, int32_t ph, int32_t pw, int64_t ao, int64_t co,
                int32_t pad_mode, ntg_affine_t aff);
/* Elementwise Dense rule and/or activation on [B, M] kernels (M spatial
 * entries per pair; spatial index m -> (a, a', c, c') of an [A, A, C, C]
 * block, or (a, c) of [A, C] when diag_spatial != 0).  var1/var2 give the
 * pre-activation variances (after the affine when has_affine). */
int ntg_affine_act(void* stream, const float* in_nngp, const float* in_ntk, float* out_nngp,
                   float* out_ntk, int64_t batch, int64_t n2, int64_t a, int64_t c,
                   int32_t diag_spatial, int32_t has_affine, ntg_affine_t aff, ntg_act_t act,
                   ntg_var_t var1, ntg_var_t var2);
/* max |x| over n entries -> out[0] (do_stabilize factor, elementwise.py:431-436). */
int ntg_max_abs(void* stream, const float* x, int64_t n, float* out);

/* ---- pooling / readout ------------------------------------------------ */
/* AvgPool / SumPool rule (linear.py:1631-1664, 3499-3572) on [B, A, A, C, C]
 * (diag_spatial = 0) or [B, A, C] (diag_spatial = 1): reduce_window with
 * window (wa, wc), strides (sa, sc), low padding (pa, pc), zero or circular
 * padding; scale = 1/prod(window) (average), 1 (sum); normalize_edges = 1
 * divides by the in-bounds window size instead. diag_spatial average pooling
 * applies the normalisation twice (linear.py:1653-1657). */
int ntg_pool(void* stream, const float* in, float* out, int64_t batch, int64_t a, int64_t c,
             int32_t wa, int32_t wc, int32_t sa, int32_t sc, int32_t pa, int32_t pc,
             int64_t ao, int64_t co, int32_t pad_mode, int32_t diag_spatial, int32_t average,
             int32_t normalize_edges);
/* Mean (average = 1) or sum over all m entries of each of B rows: [B, M] -> [B]
 * (GlobalAvgPool / GlobalSumPool, linear.py:1771-1801). `post_scale`
 * multiplies the result (1/M_extra for the diagonal-spatial case). */
int ntg_global_pool(void* stream, const float* in, float* out, int64_t batch, int64_t m,
                    int32_t average, float post_scale);
/* Flatten rule on a full-spatial kernel (linear.py:1865-1899): mean of the
 * spatial diagonal K[b, a, a, c, c] -> [B]. */
int ntg_flatten_fs(void* stream, const float* in, float* out, int64_t batch, int64_t a,
                   int64_t c);

/* ---- fused whole-network kernel per pair ------------------------------ */
/* A chain program: `nseg` spatial segments of sizes s0, s0/2, ...; segment
 * i holds nconv[i] layers of [3x3 SAME Conv + activation]; an AvgPool(2,2)
 * stride 2 separates segments; readout 0 = mean over all spatial entries
 * (GlobalAvgPool, or AvgPools down to 1x1 then Flatten), 1 = Flatten
 * (mean of the spatial diagonal). Layers are numbered in order; conv layer
 * l has affine aff[l] and activation act[l]; its pre-activation variances
 * for sample n start at var1 + n*var_stride + var_off[l] as an s_i x s_i
 * map (same for var2). */
#define NTG_CHAIN_MAX_SEG 4
#define NTG_CHAIN_MAX_LAYERS 16
typedef struct {
  int32_t nseg;
  int32_t s0;
  int32_t channels;
  int32_t readout;
  int32_t nconv[NTG_CHAIN_MAX_SEG];
  ntg_affine_t aff[NTG_CHAIN_MAX_LAYERS];
  ntg_act_t act[NTG_CHAIN_MAX_LAYERS];
  int64_t var_off[NTG_CHAIN_MAX_LAYERS];
  int64_t var_stride;
} ntg_chain_t;
/* Fused Myrtle-family kernel: inputs x1 [N1, s0, s0, K], x2 [N2, s0, s0, K]
 * (NHWC); writes the readout nngp/ntk [N1, N2] (before the layers that
 * follow the readout). Pairs (i, j) with i in [r0, r0+n1), j in [c0, c0+n2)
 * of the x1 / x2 arrays; out has row stride ld_out. Replaces the per-layer
 * chain of linear.py:1321-1424 / elementwise.py:423-477 / linear.py:1631-1664
 * / 1771-1801 / 1865-1899 for that network family. */
int ntg_chain_fwd(void* stream, const ntg_chain_t* prog, const float* x1, const float* x2,
                  int64_t r0, int64_t n1, int64_t c0, int64_t n2, const float* var1,
                  const float* var2, float* out_nngp, float* out_ntk, int64_t ld_out);
/* The same network for K(x, x), whose pairs (i, j) and (j, i) are equal: the
 * pairs (i, j) of x with itself for i in [r0, r0 + n1), j in [c0, c0 + n2) — a
 * diagonal tile (r0 == c0, n1 == n2: only i <= j evaluated) or a tile whose row
 * and column ranges are disjoint — each result written at (i, j) and (j, i) of
 * out, the whole kernel [., ld_out] (element (0, 0) at out). Half the work of
 * evaluating every pair, and an exactly symmetric output. No counterpart in the
 * reference, which evaluates every pair. */
int ntg_chain_fwd_sym(void* stream, const ntg_chain_t* prog, const float* x, int64_t r0,
                      int64_t n1, int64_t c0, int64_t n2, const float* var, float* out_q,
                      float* out_t, int64_t ld_out);

/* ---- kernel regression (predict.gradient_descent_mse, t = None) -------- */
/* Factor A = K + lambda I = L L^T in FP32 (predict.py:1224-1258 with
 * cho_factor). K is the [n, n] float32 train-train kernel; lambda =
 * diag_reg * trace(K) / n, or diag_reg when absolute != 0. L receives the
 * lower factor ([n, n], upper triangle zeroed). lambda points to two device
 * doubles: [0] receives lambda, [1] the trace of K. A non-positive pivot
 * writes its 1-based column to *info (device int, 0 = success); the caller
 * reads it back. */
int ntg_chol_factor(void* stream, const float* A, int64_t n, double diag_reg, int32_t absolute,
                    float* L, double* lambda, int* info);
/* Bytes of device workspace ntg_chol_solve needs for refinement. */
size_t ntg_chol_workspace_bytes(int64_t n, int64_t m);
/* X = (K + lambda I)^{-1} B for B [n, m]: blocked FP32 triangular solves with
 * L, then `refine_iters` steps of iterative refinement whose residual
 * B - (K + lambda I) X is accumulated in FP64 (predict.py:1235-1258 with
 * cho_solve). `workspace` must hold ntg_chol_workspace_bytes(n, m) bytes when
 * refine_iters > 0 or final_residual != NULL; final_residual (device double,
 * optional) receives max |residual| of the returned X (one more FP64 residual). */
int ntg_chol_solve(void* stream, const float* A, const float* L, const double* lambda, int64_t n,
                   const float* B, int64_t m, float* X, int32_t refine_iters, void* workspace,
                   size_t workspace_bytes, double* final_residual);

/* FP32-accurate GEMM on the tcgen05 tensor cores: C = alpha A B^T + beta C with
 * A [m, k] (row pitch lda) and B [n, k] (row pitch ldb) row-major float32, C [m, n]
 * (row pitch ldc). Each operand is split into tf32 hi + lo parts in shared memory
 * and hi hi + hi lo + lo hi are accumulated in FP32 (about 22 significant bits per
 * operand). lda and ldb multiples of 4, A and B 16-byte aligned (TMA). lower != 0
 * (m == n): only C's lower triangle (col <= row) is computed and written, the
 * symmetric rank-k update of a Cholesky factorisation. C may alias A when n <= 128.
 * Serves the trailing updates of ntg_chol_factor_tc and the solves of
 * ntg_chol_solve_tc (predict.py:1235-1258, cuSOLVER potrf/potrs in the reference). */
int ntg_gemm_tc(void* stream, const float* a, int64_t lda, const float* b, int64_t ldb, float* c,
                int64_t ldc, int64_t m, int64_t n, int64_t k, float alpha, float beta,
                int32_t lower);

/* The tensor-core Cholesky of predict.gradient_descent_mse (predict.py:1224-1258,
 * cho_factor / cho_solve): A = K + lambda I = L L^T in FP32 with 128-wide panels
 * (diagonal block factored and inverted by one CTA, the panel below as the product
 * with that inverse and the trailing update both by ntg_gemm_tc). The work runs on
 * three library streams forked from `stream` and joined back into it before the
 * call's work ends: the diagonal blocks, panels and next column block on a
 * high-priority stream, the rest of each trailing update one panel behind on a
 * second, the inverse factors below on a third. K [n, n] float32 contiguous;
 * L [n, ldl] row-major (ldl >= n, a multiple of 4, L 16-byte aligned) receives the
 * lower factor, zeros above the diagonal; lambda and info as ntg_chol_factor.
 * factor_workspace (ntg_chol_factor_tc_workspace_bytes) receives the inverses of
 * the diagonal blocks and the explicit inverse factors L^-1 and L^-T (a forward
 * block solve of L Y = I whose updates run on ntg_gemm_tc), which
 * ntg_chol_solve_tc reads. */
size_t ntg_chol_factor_tc_workspace_bytes(int64_t n, int64_t ldl);
int ntg_chol_factor_tc(void* stream, const float* A, int64_t n, double diag_reg, int32_t absolute,
                       float* L, int64_t ldl, double* lambda, int* info, void* factor_workspace,
                       size_t factor_workspace_bytes);
/* X = (K + lambda I)^{-1} B, B and X [n, m] row-major, from a factor of
 * ntg_chol_factor_tc (L itself is not read: the solves multiply by the inverse
 * factors of the factor workspace): for m <= 16 two triangular matrix-vector
 * products (two rows per warp), for more right-hand sides two ntg_gemm_tc products on
 * the transposed right-hand sides. Refinement keeps X in FP64 and accumulates the
 * products with K in double-float arithmetic (two FP32 words, about 44 significant
 * bits): for m <= 16 at most refine_iters iterations of conjugate gradients
 * preconditioned by the FP32 factor, each column stopping once its max |residual|
 * fell 1e10-fold or below 1e-15 max |b| (converges where plain refinement stalls,
 * cond(K) * u > 1); for
 * m > 16 refine_iters steps of x <- x + (L L^T)^{-1} (b - (K + lambda I) x).
 * final_residual (device double, optional) receives max |b - (K + lambda I) X| of
 * the returned X; x64_out (device double [n, m], optional) the solution before its
 * rounding to FP32, for products that keep its precision (ntg_gemm_df). B64 (device
 * double [n, m], optional): the right-hand side in FP64, whose digits beyond B's
 * float32 rounding the refinement then resolves (B still gives the first solve). */
size_t ntg_chol_solve_tc_workspace_bytes(int64_t n, int64_t m, int64_t ldl);
int ntg_chol_solve_tc(void* stream, const float* A, const float* L, int64_t ldl,
                      const void* factor_workspace, const double* lambda, int64_t n,
                      const float* B, int64_t m, float* X, int32_t refine_iters, void* workspace,
                      size_t workspace_bytes, double* final_residual, double* x64_out,
                      const double* B64);
/* Y = Y0 + A X in double-float arithmetic (two FP32 words, about 44 significant
 * bits), rounded to FP32 into Y and / or stored in FP64 into Y64 (either may be
 * NULL, not both): A [rows, n] float32 (row pitch lda), X [n, m] FP64 row-major,
 * Y0 (optional) and Y [rows, m] float32, Y64 [rows, m] double. The mean prediction
 * k_test_train (K + lambda I)^{-1} y of predict.py:236-276 and 566-745: with an
 * ill-conditioned K the product cancels, and an FP32 product of the FP32-rounded
 * solution loses cond-many digits that the FP64 solution of ntg_chol_solve_tc
 * keeps. workspace: ntg_gemm_df_workspace_bytes(rows, n, m). */
size_t ntg_gemm_df_workspace_bytes(int64_t rows, int64_t n, int64_t m);
int ntg_gemm_df(void* stream, const float* A, int64_t lda, int64_t rows, int64_t n,
                const double* X, int64_t m, const float* Y0, float* Y, double* Y64,
                void* workspace, size_t workspace_bytes);
/* log det(L L^T) of a factor of ntg_chol_factor_tc -> out[0] (device double). */
int ntg_chol_logdet_tc(void* stream, const float* L, int64_t n, int64_t ldl, double* out);

/* ---- finite-time predictions (predict.py:185-229, 860-1005, 1180-1294) ---- */
/* Eigendecomposition of the symmetric K + shift I (K [n, n] float32), the eigh of
 * the reference's _get_fns_in_eigenbasis: two-sided block Jacobi in FP32 (32-wide
 * blocks, every pair of blocks diagonalised per round by one CTA, the rotations
 * applied to K and to the eigenvectors tile by tile). Sweeps run until the
 * off-diagonal Frobenius norm is at most tol times the whole norm, or max_sweeps;
 * evals [n] (not sorted) and evecs [n, n] (column j belongs to evals[j]) are
 * written, *sweeps_out (host int, may be NULL) receives the sweeps run. Then
 * refine_steps (0-4) steps of the Ogita-Aishima refinement of all pairs, with
 * X^T X and X^T (K + shift I) X accumulated in double-float (two FP32 words): the
 * Jacobi rounds leave about 1e-5 relative error at n = 1000, a step squares it
 * down to the FP32 rounding of the output. Reads one 16-byte norm back after each
 * sweep: synchronises the stream once per sweep. */
size_t ntg_eigh_workspace_bytes(int64_t n);
int ntg_eigh(void* stream, const float* K, int64_t n, double shift, float* evals, float* evecs,
             int32_t max_sweeps, double tol, int32_t refine_steps, void* workspace,
             size_t workspace_bytes, int32_t* sweeps_out);
/* out[i, t, c] = w(lambda_i, t_t) x[i, c] for x [n, m], times t [nt] (device doubles,
 * already scaled by the learning rate) and the spectral function `kind` (pos =
 * max(lambda, 0), N = norm): 0 expm1(-pos t/N), 1 expm1(-pos t/N)/|lambda|,
 * 2 pos exp(-2 pos t/N), 3 exp(-pos t/N), 4 -expm1(-2 pos t/N)/|lambda|,
 * 5 -expm1(-pos t/N), 6 -expm1(-pos t/N)/|lambda| (predict.py:1277-1294 and the
 * ensemble covariances of :860-1005), evaluated in FP64. */
int ntg_spectral_scale(void* stream, const float* evals, const double* ts, int64_t nt, int32_t kind,
                       double norm, const float* x, int64_t n, int64_t m, float* out);

/* ---- adjoints (reverse mode; the jax.custom_vjp backward rules) -------- */
/* Derivative conventions follow the reference's custom JVPs: the square root
 * of elementwise.py:1278-1290 has derivative 0 at arguments <= 1e-30, and the
 * arctan2 of :1293-1310 divides by max(x^2 + y^2, 1e-30). */
/* VJP of the activation rule on [B, M] kernels (layout as ntg_affine_act):
 * q, t are the pre-activation nngp/ntk (t may be NULL), gq, gt the output
 * cotangents (either may be NULL); writes the cotangents of q (oq) and t (ot,
 * may be NULL) and ADDS the variance cotangents into gvar1 / gvar2 (compact
 * [n, A, C] device arrays; NULL to skip). Every kind of ntg_act_kind has an
 * adjoint; the Gelu rule is differentiated with jnp.arctan2's plain derivative,
 * as the reference writes it (elementwise.py:230-250). */
int ntg_act_bwd(void* stream, const float* q, const float* t, const float* gq, const float* gt,
                float* oq, float* ot, int64_t batch, int64_t n2, int64_t a, int64_t c,
                int32_t diag_spatial, ntg_act_t act, ntg_var_t var1, ntg_var_t var2,
                float* gvar1, float* gvar2);
/* The activation VJP of ntg_act_bwd composed with the transpose of the
 * AvgPool((2, 2), (2, 2)) that follows it (linear.py:1631-1664): the output
 * cotangents are those of the pooled kernels [B, A/2, A/2, C/2, C/2]; each entry
 * takes its window's cotangent / 16 without the [B, A, A, C, C] cotangent being
 * written. Full-spatial only, C a power of two in [4, 32], A even. No reference
 * counterpart (XLA differentiates the two layers separately). */
int ntg_act_pool_bwd(void* stream, const float* q, const float* t, const float* gq_pooled,
                     const float* gt_pooled, float* oq, float* ot, int64_t batch, int64_t n2,
                     int64_t a, int64_t c, ntg_act_t act, ntg_var_t var1, ntg_var_t var2,
                     float* gvar1, float* gvar2);
/* ntg_conv_act_fs followed by AvgPool((2, 2), (2, 2)) without the activated
 * [B, 32, 32, 32, 32] kernels being written: the conv + activation kernel leaves
 * the w-direction window sums of each plane in hp_q / hp_t (caller-provided,
 * [B, 32, 32, 16, 16]) and a second pass adds the planes into out_q / out_t
 * [B, 16, 16, 16, 16] in the summation order of ntg_pool, so the result equals
 * ntg_conv_act_fs + ntg_pool bit for bit. pre_q / pre_t receive the conv outputs
 * (the activation's VJP input). No reference counterpart (linear.py:1631-1664
 * and :1321-1424 are separate XLA ops). */
int ntg_conv_act_pool_fs(void* stream, const float* in_q, const float* in_t, float* out_q,
                         float* out_t, float* pre_q, float* pre_t, float* hp_q, float* hp_t,
                         int64_t batch, int64_t n2, int64_t a, ntg_affine_t aff, ntg_act_t act,
                         ntg_var_t var1, ntg_var_t var2);
/* First layer of a conv net on 32 x 32 images in one pass: the pair input
 * covariances of x1 [N1, 32, 32, K], x2 [N2, 32, 32, K] (1 <= K <= 4, NHWC;
 * requirements.py:542-553), the 3x3 SAME conv rule on them (linear.py:1321-1424,
 * NTK parameterisation: aff.ntk_nn = 1, ntk_c = 0, nn_scaled = 1) and the activation
 * (variances var1 / var2 of the per-sample conv outputs), without writing the
 * covariances: out_q / out_t [N1 * N2, 32, 32, 32, 32] are the activated nngp / ntk,
 * pre_q the conv output (its NTK equals it, the input NTK being zero), all as
 * ntg_input_fs followed by ntg_conv_act_fs would give them, bit for bit. */
int ntg_input_conv_act_fs(void* stream, const float* x1, const float* x2, int64_t n1,
                          int64_t n2, int64_t k, float* out_q, float* out_t, float* pre_q,
                          ntg_affine_t aff, ntg_act_t act, ntg_var_t var1, ntg_var_t var2);
/* Backward of the pair rule ntg_conv_act_fs (3x3 / stride 1 / SAME conv, W_std^2 = w2,
 * b free, followed by ABRelu) on [B, 32, 32, 32, 32] kernels, fused: the activation
 * VJP of ntg_act_bwd (pooled == 0; g_q, g_t [B, 32, 32, 32, 32] output cotangents)
 * or of ntg_act_pool_bwd (pooled != 0; g_q, g_t the AvgPool((2, 2), (2, 2)) output
 * cotangents [B, 16, 16, 16, 16]) evaluated on pre_q / pre_t (the conv outputs
 * ntg_conv_act_fs wrote), followed by the conv's transpose: writes the cotangents
 * of the conv input nngp (gin_q) and ntk (gin_t, NULL when the input NTK is the
 * zero of an input kernel) and ADDS the variance cotangents into gvar1 / gvar2
 * (compact [n, 32, 32]; NULL to skip). g_in is bit-identical to the unfused
 * ntg_act_bwd / ntg_act_pool_bwd + transposed ntg_conv_fs sequence. No reference
 * counterpart (XLA differentiates the layers separately, linear.py:1321-1424 and
 * elementwise.py:423-477). All buffers 16-byte aligned. */
int ntg_conv_act_bwd(void* stream, const float* pre_q, const float* pre_t, const float* g_q,
                     const float* g_t, int32_t pooled, float* gin_q, float* gin_t, int64_t batch,
                     int64_t n2, int64_t a, float w2, ntg_act_t act, ntg_var_t var1,
                     ntg_var_t var2, float* gvar1, float* gvar2);
/* Cotangents of the unscaled stencil sums U, Ut of an affine rule evaluated
 * as q = aff.w2 * scale * U + b2, t = ntk_w2 * scale * Ut + ... (n entries). */
int ntg_affine_bwd(void* stream, const float* gq, const float* gt, float* gu, float* gut,
                   int64_t n, ntg_affine_t aff, float scale);
/* Hyperparameter cotangent sums of an NTK-parameterised affine rule from its
 * outputs (q, t) and their cotangents: out[0] += d/d(W^2), out[1] += d/d(b^2)
 * (two device doubles, accumulated). */
int ntg_affine_hyper_bwd(void* stream, const float* q, const float* t, const float* gq,
                         const float* gt, int64_t n, float w2, float b2, double* out);
/* Transpose of the Conv stencil sum (full spatial [B, A, A, C, C] or diagonal
 * spatial [B, A, C]): geometry as ntg_conv_fs. */
int ntg_stencil_bwd(void* stream, const float* gu, float* gin, int64_t batch, int64_t a,
                    int64_t c, int32_t fh, int32_t fw, int32_t sh, int32_t sw, int32_t ph,
                    int32_t pw, int64_t ao, int64_t co, int32_t pad_mode, int32_t diag_spatial);
/* Transpose of ntg_pool (windows up to 6 per axis). */
int ntg_pool_bwd(void* stream, const float* gout, float* gin, int64_t batch, int64_t a, int64_t c,
                 int32_t wa, int32_t wc, int32_t sa, int32_t sc, int32_t pa, int32_t pc,
                 int64_t ao, int64_t co, int32_t pad_mode, int32_t diag_spatial, int32_t average,
                 int32_t normalize_edges);
/* Transpose of the readouts: gin[b, m] = gout[b] * scale on all m entries
 * (global pooling) or only on the spatial diagonal (flatten_fs = 1, Flatten). */
int ntg_readout_bwd(void* stream, const float* gout, float* gin, int64_t batch, int64_t a,
                    int64_t c, int32_t flatten_fs, int64_t m, float scale);
/* Image cotangents through ntg_input_fs: ADDS into gx [nself, A, C, K]; side 0
 * treats the cotangent g as indexed by (self, other) pairs, side 1 as
 * (other, self); n2 == 0 for the per-sample covariance (pairs (i, i)). */
int ntg_input_fs_bwd(void* stream, const float* g, const float* x_other, float* gx,
                     int64_t nself, int64_t nother, int64_t n2, int64_t a, int64_t c, int64_t k,
                     int32_t side);
/* Both image cotangents of the full-spatial input covariance in one pass over
 * its cotangent g (requirements.py:641-830, the _cov of an image pair): gx1 +=
 * dG/dx1 contracted with g, gx2 += dG/dx2 (pairs g [N1, N2, A, A, C, C]); with
 * n2 == 0 the per-sample covariances g [N1, A, A, C, C] of x1 with itself, both
 * terms into gx1 (x2, gx2 unused). Equivalent to the two side calls of
 * ntg_input_fs_bwd. */
int ntg_input_fs_bwd2(void* stream, const float* g, const float* x1, const float* x2,
                      float* gx1, float* gx2, int64_t n1, int64_t n2, int64_t a, int64_t c,
                      int64_t k);
/* Adjoint of ntg_input_ds, ADDING into gx1 [N1, P, K] and gx2 [N2, P, K]:
 * pairs g [N1, N2, P] (gx2 may be gx1 when x2 is x1), or with n2 == 0 the
 * per-sample covariances g [N1, P] of x1 (x2, gx2 unused). */
int ntg_input_ds_bwd(void* stream, const float* g, const float* x1, const float* x2,
                     float* gx1, float* gx2, int64_t n1, int64_t n2, int64_t p, int64_t k);
/* C [m, n] (+)= alpha op(A) B, op(A) = A [m, k] or, trans_a != 0, A^T with A [k, m]
 * (flat Gram adjoint). */
int ntg_gemm_ex(void* stream, const float* a, const float* b, float* c, int64_t m, int64_t n,
                int64_t k, int32_t trans_a, float alpha, int32_t accumulate);
/* dst[i*s_n + a*s_a + c*s_c] += src[i, a, c]: folds variance cotangents
 * [n, A, C] into the diagonal of a per-sample kernel cotangent. */
int ntg_diag_add(void* stream, const float* src, float* dst, int64_t n, int64_t a, int64_t c,
                 int64_t s_n, int64_t s_a, int64_t s_c);
/* gx [n, d] += 2 gcov[i] x[i, :] / d (adjoint of ntg_cov_diag). */
int ntg_cov_diag_bwd(void* stream, const float* gcov, const float* x, float* gx, int64_t n,
                     int64_t d);

/* log det(L L^T) = 2 sum log L_ii of a factor from ntg_chol_factor -> out[0]. */
int ntg_chol_logdet(void* stream, const float* L, int64_t n, double* out);
/* Cotangent of the Gaussian-process negative log-likelihood
 * 1/2 tr(Y^T A^{-1} Y) + m/2 log det A + const with A = K + lambda I:
 * out = g (-1/2 alpha alpha^T + m/2 A^{-1}) (alpha = A^{-1} Y [n, m], kinv = A^{-1}),
 * plus reg_over_n * trace(out) on the diagonal when lambda = diag_reg trace(K) / n
 * (reg_over_n = diag_reg / n; 0 for an absolute regulariser). tr: device double. */
int ntg_nll_grad(void* stream, const float* kinv, const float* alpha, int64_t n, int64_t m,
                 float g, double reg_over_n, float* out, double* tr);

/* No counterpart in the reference. ntg_chol_solve without a caller workspace,
 * for callers that cannot allocate device memory where they call the solve
 * (an XLA FFI handler, which only receives the buffers XLA allocated for it;
 * a server that reserved all device memory up front for its own pool). The refinement workspace is a fixed device array of
 * NTG_NOALLOC_SCRATCH_BYTES owned by the library: each GPU that loads the
 * library holds it until the process exits, and the call fails with
 * NTG_ERR_INVALID_ARG when ntg_chol_workspace_bytes(n, m) exceeds it (about
 * n * m <= 87,000). The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress) and caches it per device ordinal; make that
 * first call before any stream capture. The cached address belongs to the
 * device's primary context (the one the CUDA runtime and PyTorch use): it is
 * not valid in another context made current through the driver API, nor after
 * cudaDeviceReset. n must be at most 46340 (the factorisation's limit) and
 * n * m at most (NTG_NOALLOC_SCRATCH_BYTES - 256) / 12; both are checked before
 * any size is computed. All calls share the array: calls that overlap on the
 * GPU (other streams, other threads) race and must be serialised by the caller. No
 * cudaMalloc, cudaFree or allocating library routine is called. Arguments
 * and results are those of ntg_chol_solve. */
#define NTG_NOALLOC_SCRATCH_BYTES (1u << 20)
int ntg_chol_solve_noalloc(void* stream, const float* A, const float* L, const double* lambda,
                           int64_t n, const float* B, int64_t m, float* X, int32_t refine_iters,
                           double* final_residual);

#ifdef __cplusplus
}
#endif

#endif /* NT_GB300_H_ */
