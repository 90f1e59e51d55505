/*
 * matfree_gb300 — C ABI of the GB300 (sm_103a) stochastic Lanczos quadrature path.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*; NULL is the legacy default stream), returns an int status
 * (MFG_OK == 0) and allocates no device memory: the caller owns every buffer,
 * including the workspace whose size mfg_slq_workspace_bytes() reports.
 * Calls on different streams with different workspaces may run concurrently.
 *
 * Memory layout ("probe-major panels"): a set of p vectors of length n is
 * stored as p rows of ld elements (ld >= n, ld % 8 == 0, 16-byte aligned
 * base).  The Krylov basis of p probes with k vectors each is p x k rows of ld
 * elements (probe b, vector i at row b*k + i).  Hessenberg matrices are p
 * row-major k x k float64 blocks (column j holds step j's projection
 * coefficients and, below the diagonal, the norm of the new vector).
 *
 * The reference (pnkraemer/matfree) is JAX; the functions each entry point
 * stands in for are cited file:line relative to that project.
 */
#ifndef MATFREE_GB300_H
#define MATFREE_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define MFG_API __attribute__((visibility("default")))
#else
#define MFG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  MFG_OK = 0,
  MFG_ERR_BAD_ARG = 1,     /* a size, pointer, alignment or flag is invalid   */
  MFG_ERR_RANGE = 2,       /* num_matvecs outside [0, n] ("exceeds")          */
  MFG_ERR_WORKSPACE = 3,   /* workspace smaller than mfg_slq_workspace_bytes  */
  MFG_ERR_CUDA = 4,        /* a CUDA runtime/driver call failed               */
  MFG_ERR_UNSUPPORTED = 5, /* combination not implemented (e.g. op/precision) */
  MFG_ERR_NO_CONVERGENCE = 6, /* tridiagonal eigensolver hit its sweep limit  */
  MFG_ERR_TIMEOUT = 7,     /* a bounded device-side wait gave up             */
  MFG_ERR_SCRATCH_LIMIT = 8, /* problem larger than a fixed static scratch    */
  MFG_ERR_RETRY = 9         /* two-sweep reorthogonalisation lost accuracy:   */
                            /* repeat the call with reortho = 1               */
};

/* ---- element type of vectors and bases --------------------------------- */
enum { MFG_F32 = 0, MFG_F64 = 1 };

/* ---- operator descriptors ---------------------------------------------- */
enum {
  MFG_OP_DENSE = 0,    /* row-major n x n matrix, see precision below          */
  MFG_OP_CSR = 1,      /* CSR, int32 row_ptr/col_idx, float32 values           */
  MFG_OP_CALLBACK = 2  /* caller-supplied apply(V -> W) on device panels        */
};

enum {
  MFG_PREC_FP32 = 0,   /* dense float32 matrix, float32 CUDA-core product      */
  MFG_PREC_BF16 = 1,   /* dense bf16 matrix (a), tcgen05 bf16 x bf16 -> fp32   */
  MFG_PREC_BF16X3 = 2, /* bf16 hi (a) + lo (a_lo); hi*hi + hi*lo + lo*hi       */
  MFG_PREC_FP64 = 3    /* dense float64 matrix and float64 basis               */
};

/* W = A V for a probe-major panel V (p rows of ld), all on `stream`. */
typedef int (*mfg_apply_fn)(void *ctx, const void *V, void *W, int64_t n,
                            int64_t p, int64_t ld, void *stream);

typedef struct mfg_operator {
  int32_t kind;      /* MFG_OP_*                                              */
  int32_t precision; /* MFG_PREC_* (dense); MFG_PREC_FP32 for CSR/callback    */
  int64_t n;         /* dimension                                             */
  const void *a;     /* dense: matrix (fp32/fp64/bf16-hi), lda elements/row   */
  const void *a_lo;  /* dense BF16X3: bf16 low part, same lda                 */
  int64_t lda;
  const int32_t *row_ptr; /* CSR: n + 1 entries                               */
  const int32_t *col_idx; /* CSR: nnz entries                                 */
  const float *values;    /* CSR: nnz entries                                 */
  int64_t nnz;
  double shift;      /* the operator applied is A + shift * I                 */
  mfg_apply_fn apply;/* callback operators                                    */
  void *ctx;
} mfg_operator;

/* ---- matrix functions of the quadrature -------------------------------- */
enum {
  MFG_FUN_LOG = 0,  /* f(x) = log(x)                        (funm.py:199)    */
  MFG_FUN_EXP = 1,  /* f(x) = exp(param * x)                                 */
  MFG_FUN_POW = 2,  /* f(x) = x ** param                                     */
  MFG_FUN_NONE = 3  /* eigenvalues and first components only                 */
};

/* Library version (major*10000 + minor*100 + patch). */
MFG_API int mfg_version(void);

/* Human-readable text of a status code; never NULL. */
MFG_API const char *mfg_status_string(int status);

/* Where and why the most recent MFG_ERR_CUDA on the calling host thread
 * arose ("file:line: CUDA error text"); empty if none.  Never NULL. */
MFG_API const char *mfg_last_error(void);

/* Bytes of workspace the SLQ / tridiagonalisation entry points need. */
MFG_API size_t mfg_slq_workspace_bytes(const mfg_operator *op, int64_t k, int64_t p, int64_t ld);

/* Probe sampler: Rademacher +-1 (Philox4x32-10, key = 2 words) written as a
 * probe-major panel of `dtype` (MFG_F32/MFG_F64); padding columns set to 0.
 * Replaces stochtrace.sampler_signs (matfree/stochtrace.py:932-937,974-977)
 * and backend/prng.py:26-29. */
MFG_API int mfg_sampler_signs(const uint32_t key[2], int64_t num, int64_t n, int64_t ld,
                      int32_t dtype, void *out, void *stream);

/* Probe sampler: standard normal (Box-Muller on Philox words).
 * Replaces stochtrace.sampler_normal (matfree/stochtrace.py:927-929). */
MFG_API int mfg_sampler_normal(const uint32_t key[2], int64_t num, int64_t n, int64_t ld,
                       int32_t dtype, void *out, void *stream);

/* W = (A + shift I) V for a probe-major panel; the batched `matvec(v)` that
 * matfree evaluates under vmap (matfree/decomp.py:460, stochtrace.py:49). */
MFG_API int mfg_operator_apply(const mfg_operator *op, const void *V, void *W, int64_t p,
                       int64_t ld, void *workspace, size_t workspace_bytes, void *stream);

/* Batched Arnoldi with classical Gram-Schmidt applied twice over the p
 * columns of V (probe-major, dtype F64 for MFG_PREC_FP64 else F32):
 * Q (p*k rows of ld), H (p k x k float64), residual (p rows of ld) and
 * init_len_inv[p] = 1/||v_b||.
 * Replaces decomp.tridiag_sym(k, reortho="full") / decomp.hessenberg
 * (matfree/decomp.py:30-152, 353-477).  reortho: 1 = "full" (Gram-Schmidt
 * twice against all vectors), 0 = "none" of hessenberg (once against all
 * vectors), 2 = three-term Lanczos of tridiag_sym(reortho="none")
 * (decomp.py:215-291: H holds a_j on the diagonal and b_j below it),
 * 3 = "full" in two basis reads per step (see MFG_SLQ_TWO_SWEEP; falls back
 * to 1 outside float bases with 2 <= k <= 129; workspace from
 * mfg_slq_ex_workspace_bytes(..., MFG_SLQ_TWO_SWEEP); check
 * mfg_workspace_status for MFG_ERR_RETRY). */
MFG_API int mfg_hessenberg(const mfg_operator *op, int64_t k, int64_t p, const void *V,
                   int64_t ld, int32_t reortho, void *Q, double *H, void *residual,
                   double *init_len_inv, void *workspace, size_t workspace_bytes,
                   void *stream);

/* Bytes of workspace mfg_hessenberg_adjoint needs. */
MFG_API size_t mfg_adjoint_workspace_bytes(const mfg_operator *op, int64_t k, int64_t p, int64_t ld);

/* Reverse pass of mfg_hessenberg for p probes (the Hessenberg adjoint of
 * Kraemer et al. 2024) with cotangents dH (p k x k float64), optional dr
 * (p rows of ld) and dc (p float64); the cotangent of Q must be zero, which
 * holds for every integrand that reads only T.  Inputs are the forward
 * outputs Q, H, residual and init_len_inv.  Outputs: dv (p rows of ld), the
 * cotangent of the starting vectors, and Lambda (p*k rows of ld, layout of
 * Q), the adjoint states lambda_idx of every step, from which the caller
 * forms parameter gradients sum_idx lambda_idx^T (dA/dtheta) q_idx.  The
 * operator must be symmetric (A^T lambda is evaluated as A lambda).
 * Replaces decomp._hessenberg_adjoint / _hessenberg_adjoint_step
 * (matfree/decomp.py:480-600); k = 0 returns MFG_ERR_RANGE (decomp.py:483-486). */
MFG_API int mfg_hessenberg_adjoint(const mfg_operator *op, int64_t k, int64_t p, int64_t ld,
                                   const void *Q, const double *H, const void *residual,
                                   const double *init_len_inv, const double *dH, const void *dr,
                                   const double *dc, void *Lambda, void *dv, void *workspace,
                                   size_t workspace_bytes, void *stream);

/* mfg_hessenberg_adjoint with a cotangent of the basis as well: dQ (p*k
 * rows of ld, layout of Q; NULL means zero) enters through Pi_xi = dQ^T +
 * gamma r^T and Pi_gamma = ... - dQ^T Q (matfree/decomp.py:505-506, used by
 * the reverse step at :592-599).  Every integrand that reads Q -- f(A) v by
 * Lanczos (funm.py:114-147) -- needs it.  Same workspace and outputs as
 * mfg_hessenberg_adjoint, which is this call with dQ = NULL. */
MFG_API int mfg_hessenberg_adjoint_ex(const mfg_operator *op, int64_t k, int64_t p, int64_t ld,
                                      const void *Q, const double *H, const void *residual,
                                      const double *init_len_inv, const void *dQ, const double *dH,
                                      const void *dr, const double *dc, void *Lambda, void *dv,
                                      void *workspace, size_t workspace_bytes, void *stream);

/* Tile configuration of the bf16 / bf16x3 tensor-core operator product (the
 * CTA-pair form, n >= 1024) for operators of n in [n_lo, n_hi] applied to
 * p in [p_lo, p_hi] probe vectors: probe tiles of bn columns (a multiple of
 * 32 in [64, 256]; narrower tiles give more tiles per operator and re-read it
 * once per tile) and the form split_k: 1 one tile per CTA pair, 2 K split in
 * two halves on twice the pairs, 3 persistent pairs (one per two SMs) that
 * spread the last wave of tiles over every SM by splitting each of its tiles
 * once along K (0 and bn = 0 keep the built-in choice).  Split tiles add two
 * partial products into a zeroed output, which does not depend on timing.  The last matching rule applies; process-wide, at most
 * 256 rules.  Written by matfree_gb300.tuning (an autotuner that times the
 * candidates on the device); no counterpart in the reference. */
MFG_API int mfg_gemm_tuning_add(int64_t n_lo, int64_t n_hi, int64_t p_lo, int64_t p_hi, int32_t bn,
                                int32_t split_k);
MFG_API int mfg_gemm_tuning_clear(void);

/* Work list of the persistent CTA-pair form (mfg_gemm_tuning_add split_k =
 * 3) of an n x n operator applied to p probes with probe tiles of bn columns
 * on at most max_pairs CTA pairs (half the SMs), K tails shorter than
 * min_tail slices of 32 not split off (the product uses its ring depth).
 * Writes up to `capacity` items of four int32 (pair, tile, first K slice,
 * end K slice) in the order each pair runs them, tiles numbered row tile
 * (256 rows) first; returns the number of items, or minus an error code.
 * Host only (no device call): for inspecting and testing the schedule. */
MFG_API int64_t mfg_gemm_pair_schedule(int64_t n, int64_t p, int32_t bn, int32_t max_pairs,
                                       int32_t min_tail, int32_t *items, int64_t capacity);

/* out_b = sum_i coef[b][i] q_{b,i} for p Krylov bases Q (p*k rows of ld,
 * dtype MFG_F32/MFG_F64; coef p x k float64): the back-projection
 * Q^T (f(T) e1) of f(A) v by Lanczos (matfree/funm.py:142-146), batched.
 * Columns n..ld-1 of out are set to zero. */
MFG_API int mfg_basis_combine(int32_t dtype, int64_t k, int64_t p, int64_t n, int64_t ld,
                              const void *Q, const double *coef, void *out, void *stream);

/* Eigenvalues (ascending, eigvals p x k) and every eigenvector (eigvecs p
 * k x k, row-major, column j = eigenvector j) of the symmetric tridiagonal
 * part of (H + H^T)/2 for p Hessenberg matrices, in float64: divide and
 * conquer (one CTA per problem) for 16 <= k <= 64, implicit QL (one warp per
 * problem) otherwise; scratch holds p k x k doubles (used by the QL form).
 * The dense eigh that the derivative of e1^T f(T) e1 uses
 * (matfree/funm.py:322-335 under autodiff). */
MFG_API int mfg_tridiag_eigh(int64_t k, int64_t p, const double *H, double *eigvals,
                             double *eigvecs, double *scratch, void *stream);

/* For each of p Hessenberg matrices: T = (H + H^T)/2 restricted to its
 * tridiagonal part, its eigenvalues and the squares of the first eigenvector
 * components in float64 -- divide and conquer for 16 <= k <= 2048, implicit
 * QL with the first components tracked (Golub-Welsch) otherwise -- and
 * values[b] = scale[b] * sum_i f(lambda_i) s_1i^2.  eigvals / first_sq may be
 * NULL; scale may be NULL (1).
 * Replaces funm.dense_funm_sym_eigh + the quadform's e1^T f(T) e1
 * (matfree/funm.py:239-241, 322-335) and decomp.py:133-135. */
MFG_API int mfg_tridiag_quadrature(int64_t k, int64_t p, const double *H, int32_t fun,
                           double param, const double *scale, double *values,
                           double *eigvals, double *first_sq, void *stream);

/* The whole SLQ integrand for p probes: ||v_b||^2 e1^T f(T_b) e1 with
 * T_b from mfg_hessenberg(reortho="full") of v_b/||v_b||.  values[p] and
 * mean_sem[2] = (mean, std/sqrt(p)) are device float64 (mean_sem may be NULL).
 * Replaces estimator_monte_carlo(monte_carlo_funm_sym(dense_funm_sym_eigh(f),
 * tridiag_sym(k)), sampler) (matfree/stochtrace.py:47-50,82-87;
 * funm.py:186-241).  Q, H may be NULL: the basis then lives in the workspace
 * and is not returned. */
MFG_API int mfg_slq(const mfg_operator *op, int64_t k, int64_t p, const void *probes,
            int64_t ld, int32_t fun, double param, double *values, double *mean_sem,
            void *Q, double *H, void *workspace, size_t workspace_bytes, void *stream);

/* mfg_slq with options.  MFG_SLQ_TWO_SWEEP: the same full reorthogonalisation
 * in two reads of the Krylov basis per step instead of three (the second
 * projection of step j-1 is done together with the first projection of step
 * j, and A q_j is recovered from A applied to the not yet reorthogonalised
 * vector through the Arnoldi relation).  H, and so values, equal mfg_slq's to
 * rounding.  Applies to float bases with 2 <= k <= 129 (otherwise the call
 * runs mfg_slq).  When a step's second projection exceeds 0.1 of the vector
 * (a vector left largely inside the basis by one projection, near an
 * invariant subspace) the rounding of the recovered product is no longer
 * negligible: the run then records MFG_ERR_RETRY in the workspace, read back
 * with mfg_workspace_status, and the caller repeats the call without the
 * flag.  Workspace: mfg_slq_ex_workspace_bytes with the same flags. */
enum { MFG_SLQ_TWO_SWEEP = 1 };
MFG_API size_t mfg_slq_ex_workspace_bytes(const mfg_operator *op, int64_t k, int64_t p, int64_t ld,
                                          int32_t flags);
MFG_API int mfg_slq_ex(const mfg_operator *op, int64_t k, int64_t p, const void *probes,
                       int64_t ld, int32_t fun, double param, double *values, double *mean_sem,
                       void *Q, double *H, int32_t flags, void *workspace,
                       size_t workspace_bytes, void *stream);

/* Waits for `stream` and returns the device-side status of the last
 * mfg_slq / mfg_slq_ex / mfg_hessenberg run on this workspace: MFG_OK,
 * MFG_ERR_RETRY, MFG_ERR_NO_CONVERGENCE or MFG_ERR_TIMEOUT (the host return
 * code of the call reports launch-time errors only). */
MFG_API int mfg_workspace_status(const void *workspace, void *stream);

/* Dense RBF kernel matrix K_ij = s2 exp(-|x_i - x_j|^2 / (2 ell^2)) from
 * points x (n x dim float32, row-major), WITHOUT the nugget (pass tau as the
 * operator shift).  precision selects the storage: FP32 -> a (float),
 * BF16 -> a (bf16), BF16X3 -> a (bf16 hi) and a_lo (bf16 lo), FP64 -> a
 * (double).  Stands in for the user covariance closure of
 * tutorials/8_gaussian_logpdf.py:21-30. */
MFG_API int mfg_rbf_build(const float *x, int64_t n, int32_t dim, double s2, double ell,
                  int32_t precision, void *a, void *a_lo, int64_t lda, void *stream);

/* The derivative of the same matrix with respect to log(ell):
 * s2 exp(-|x_i - x_j|^2 / (2 ell^2)) |x_i - x_j|^2 / ell^2, same storage
 * options; the operator that contracts adjoint states for d logdet / d log ell
 * (the parameter part of the matvec VJP in matfree/decomp.py:587-589). */
MFG_API int mfg_rbf_build_dlogell(const float *x, int64_t n, int32_t dim, double s2, double ell,
                                  int32_t precision, void *a, void *a_lo, int64_t lda, void *stream);

/* Split a float32 matrix into bf16 hi = bf16(a) and lo = bf16(a - hi). */
/* ---- Golub-Kahan bidiagonalisation and product quadrature --------------- */

/* Workspace bytes of mfg_bidiag / mfg_slq_product (0 on bad arguments). */
MFG_API size_t mfg_bidiag_workspace_bytes(const mfg_operator *A, const mfg_operator *At, int64_t k,
                                          int64_t p, int64_t ld);

/* decomp.bidiag(k, reortho="full") (matfree/decomp.py:641-750) from every
 * probe-major row of V0: A V ~ U B, A^T U = V B^T + residual e_k^T, with the
 * operator A and its transpose At (both n x n; pad rectangular maps with
 * zeros).  U, V: (p, k, ld) left / right vectors; alphas, betas: (p, k)
 * float64 with B = diag(alphas) + superdiag(betas[:, 1:]) and betas[:, 0] =
 * 0; residual (p, ld) = beta_k v_k; init_len_inv (p) = 1 / ||v0||.  Every
 * vector is reorthogonalised twice (classical Gram-Schmidt) against the
 * vectors of its side.  residual and init_len_inv may be NULL. */
MFG_API int mfg_bidiag(const mfg_operator *A, const mfg_operator *At, int64_t k, int64_t p,
                       const void *V0, int64_t ld, void *U, void *V, double *alphas,
                       double *betas, void *residual, double *init_len_inv, void *workspace,
                       size_t workspace_bytes, void *stream);

/* funm.monte_carlo_funm_product(dense_funm_product_svd(f), bidiag(k))
 * (matfree/funm.py:246-320) on every probe row: values[b] = ||v_b||^2
 * e1^T f(B_b^T B_b) e1 with f = log (product log-determinant) or x ** param
 * (Schatten norms: param = power / 2); mean_sem (2 doubles, may be NULL). */
MFG_API int mfg_slq_product(const mfg_operator *A, const mfg_operator *At, int64_t k, int64_t p,
                            const void *probes, int64_t ld, int32_t fun, double param,
                            double *values, double *mean_sem, void *workspace,
                            size_t workspace_bytes, void *stream);

/* ---- conjugate gradients ------------------------------------------------ */

/* Workspace bytes of mfg_cg for p right-hand sides (0 on bad arguments). */
MFG_API size_t mfg_cg_workspace_bytes(const mfg_operator *op, int64_t p, int64_t ld);

/* Solve (A + shift I) X = B for each of the p probe-major rows of B (ld
 * elements apart) by conjugate gradients from X = 0 without preconditioner,
 * as jax.scipy.sparse.linalg.cg (used by matfree's Gaussian log-pdf,
 * tutorials/8_gaussian_logpdf.py:50): a row stops once ||r||^2 <=
 * max(tol^2 ||b||^2, atol^2) or after maxiter iterations (maxiter <= 0:
 * 10 n), and stays unchanged while the other rows iterate.  iters (device,
 * p int32, may be NULL) receives the iterations each row ran.  Synchronises
 * `stream` every 8 iterations to test whether any row still runs (finished
 * rows stay unchanged meanwhile); returns the first device-side error status
 * (e.g. MFG_ERR_TIMEOUT) or MFG_OK. */
MFG_API int mfg_cg(const mfg_operator *op, int64_t p, const void *B, void *X, int64_t ld,
                   double tol, double atol, int64_t maxiter, int32_t *iters, void *workspace,
                   size_t workspace_bytes, void *stream);

/* ---- launch accounting (diagnostics) ------------------------------------ */
enum {
  MFG_PROF_APPLY = 0,  /* operator application (GEMM / SpMM / callback)        */
  MFG_PROF_PROJ = 1,   /* Gram-Schmidt projections Q^T w                        */
  MFG_PROF_SUB = 2,    /* Gram-Schmidt updates w -= Q h (and norms)             */
  MFG_PROF_SCALE = 3,  /* normalisation (+ bf16 split of the new vector)        */
  MFG_PROF_QUAD = 4,   /* tridiagonal eigensolve + quadrature + mean            */
  MFG_PROF_OTHER = 5,  /* samplers, operator builds, initial norms              */
  MFG_PROF_SUBPROJ = 6, /* fused update + second projection (one basis read)   */
  MFG_PROF_CLASSES = 7
};

/* Reset the process-wide launch counters; timing != 0 also brackets every
 * launch with CUDA events on its stream (for benchmarks; not thread-safe with
 * respect to concurrent readers). */
MFG_API int mfg_profile_enable(int timing);

/* Per class: summed event time (ms), algorithmic bytes and flops of the timed
 * launches, and the number of launches since the last reset.  Synchronises
 * on the recorded events.  Any output pointer may be NULL. */
MFG_API int mfg_profile_read(int32_t nclasses, double *ms, double *bytes, double *flops,
                             int64_t *launches);

MFG_API int mfg_split_bf16(const float *a, int64_t rows, int64_t cols, int64_t lda,
                   void *hi, void *lo, int64_t ld_out, void *stream);

/* Operator application that allocates nothing: the same W = (A + shift I) V
 * as mfg_operator_apply, for callers that cannot allocate device memory and
 * therefore cannot provide a workspace -- code running inside another
 * framework's fixed memory pool (where a second allocator would fight the
 * pool's own accounting), or an embedded host without a device allocator.
 * It has no counterpart in the reference (matfree is JAX and never manages
 * device memory itself).
 *
 * The only scratch it needs lives in one fixed array inside this library:
 * MFG_NOALLOC_SCRATCH_BYTES (32 MiB) of device memory that every GPU which
 * loads the library holds until the process exits.  Its layout is a 256-byte
 * status word, then the bf16 hi copy of the panel, then (bf16x3) the bf16 lo
 * copy, each copy padded to a multiple of 256 bytes.  A call is rejected with
 * MFG_ERR_SCRATCH_LIMIT, before any work is queued, when
 *     256 + copies * round_up(p * ld * 2, 256) > MFG_NOALLOC_SCRATCH_BYTES
 * with copies = 2 for MFG_PREC_BF16X3, 1 for MFG_PREC_BF16 and 0 otherwise
 * (fp32, fp64 and CSR need no panel copy and are never rejected for size).
 * The first call on a device looks up that device's copy of the array (no
 * allocation); make that first call before any stream capture.  All calls
 * share the one array and the status word is cleared at the start of each
 * call: calls that overlap on the GPU (other streams, other threads) race on
 * it and must be serialised by the caller.
 *
 * The return code reports launch-time errors only.  A bounded device-side
 * wait that gives up (MFG_ERR_TIMEOUT; the product is then left incomplete)
 * is recorded in the status word and is otherwise silent: read it with
 * mfg_operator_apply_noalloc_status. */
#define MFG_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
MFG_API int mfg_operator_apply_noalloc(const mfg_operator *op, const void *V, void *W,
                                       int64_t p, int64_t ld, void *stream);

/* Waits for `stream` and returns the device-side status of the most recent
 * mfg_operator_apply_noalloc on the current device (MFG_OK or
 * MFG_ERR_TIMEOUT), or a host error code.  Allocates nothing. */
MFG_API int mfg_operator_apply_noalloc_status(void *stream);

/* Self-test of the bounded device-side waits that every kernel of this
 * library uses (failure detection without a GPU fault).  One CTA waits on an
 * mbarrier that nothing arrives on: warp 0 polls for `limit_ns`, gives up,
 * raises the CTA's failure flag and writes MFG_ERR_TIMEOUT to *status (a
 * device int32 the caller zeroes); warp 1 sleeps in the wait with the
 * production limit (2 s) and leaves early through the failure flag.  `times`
 * (device, 5 x uint64) receives: warp 0's wait in ns, whether it completed
 * (0), warp 1's wait in ns, whether it completed (0), the final flag (1).
 * No copy is in flight and no tensor memory is held, so the context stays
 * usable; the return code reports launch errors only.  No reference
 * counterpart: matfree's JAX code has no device-side waits. */
MFG_API int mfg_wait_selftest(uint64_t limit_ns, void *status, void *times, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MATFREE_GB300_H */
