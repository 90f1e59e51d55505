// Host-side launchers of the matfree_gb300 kernels (internal interface).
#pragma once

#include "common.cuh"

namespace mfg {

// lanczos_kernels.cu
template <typename T>
int launch_sampler(int stream_id, uint32_t k0, uint32_t k1, int64_t num, int64_t n, int64_t ld,
                   T *out, cudaStream_t s);
template <typename T> int64_t num_chunks(int64_t n);
template <typename T>
int launch_proj(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols, const T *Wv,
                int64_t w_bstride, int64_t n, int64_t p, double *partials, unsigned *counters,
                double *out, int64_t out_bstride, int64_t out_istride, cudaStream_t s,
                int *status = nullptr);
template <typename T>
int launch_sub(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols, const double *coef,
               int64_t c_bstride, int64_t c_istride, const T *Win, T *Wout, int64_t w_bstride,
               int64_t n, int64_t p, bool with_norm, bool store, double *partials,
               unsigned *counters, double *norm_out, double *norm_out2, int64_t norm2_bstride,
               cudaStream_t s, int *status = nullptr);
template <typename T> int sub_proj_rows_per_thread(int ncols);
template <typename T> int64_t max_fused_chunks(int64_t n);
template <typename T>
int launch_sub_proj(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols, const double *coef,
                    int64_t c_bstride, int64_t c_istride, T *Wv, int64_t w_bstride, int64_t n,
                    int64_t p, double *partials, unsigned *counters, double *out,
                    int64_t out_bstride, int *status, cudaStream_t s);
template <typename T>
int launch_scale(const T *Win, int64_t w_bstride, int64_t n, int64_t p, const double *norm, T *out,
                 int64_t out_bstride, __nv_bfloat16 *hi, __nv_bfloat16 *lo, int64_t bf_bstride,
                 cudaStream_t s);
int launch_inv(const double *x, double *y, int64_t p, cudaStream_t s);
// two-sweep Arnoldi step (lanczos_kernels.cu; float bases).  One two-vector
// pass covers at most kTwoSweepPassCols basis vectors (both vectors' sums stay
// in registers); steps with more run it on column blocks.  k <= kTwoSweepMaxK.
constexpr int kTwoSweepPassCols = 64;
constexpr int kTwoSweepMaxK = 129;
template <typename T>
int launch_proj2(const T *Q, int64_t q_bstride, int64_t q_istride, int coff, int ncols,
                 const T *Wa, const T *Wb, int64_t w_bstride, int64_t n, int64_t p,
                 double *partials, unsigned *counters, double *out, int64_t out_bstride,
                 int64_t koff, double *cross, int64_t cross_bstride, int *status, cudaStream_t s);
template <typename T>
int launch_sub2(const T *Q, int64_t q_bstride, int64_t q_istride, int coff, int ncols,
                const double *coef, int64_t c_bstride, int64_t koff, T *Wa, int64_t wa_bstride,
                const T *Wb, int64_t wb_bstride, T *Wo, int64_t wo_bstride, int64_t n, int64_t p,
                double *partials, unsigned *counters, double *dots, int *status, cudaStream_t s);
int launch_twosweep_coef(int j, int k, int64_t p, const double *X2, int64_t koff,
                         const double *dots, double *H, double *Hh, double *nu, double *cf,
                         int *status, cudaStream_t s);
template <typename T>
int launch_twosweep_finish(T *Qj, int64_t q_bstride, const T *Z, int64_t w_bstride, int64_t n,
                           int64_t p, const double *cf, T *qt, __nv_bfloat16 *hi,
                           __nv_bfloat16 *lo, int64_t bf_bstride, cudaStream_t s);
// conjugate gradients on probe-major panels (lanczos_kernels.cu)
template <typename T>
int launch_cg_init(const T *B, T *X, T *R, T *P, int64_t ld, int64_t n, int64_t p,
                   __nv_bfloat16 *hi, __nv_bfloat16 *lo, double *partials, unsigned *counters,
                   double tol2, double atol2, double *rs, double *thr, int *iters, cudaStream_t s);
template <typename T>
int launch_cg_update(T *X, T *R, const T *P, const T *W, int64_t ld, int64_t n, int64_t p,
                     const double *rs, const double *pap, const double *thr, double *partials,
                     unsigned *counters, double *rs_next, int *nactive, int *nactive_clear,
                     int *iters, cudaStream_t s);
// one CTA per probe for the whole post-product iteration of vectors up to kCgSmallMaxN
constexpr int64_t kCgSmallMaxN = 8192;
template <typename T>
int launch_cg_step_small(T *X, T *R, T *P, const T *W, int64_t ld, int64_t n, int64_t p,
                         const double *rs, const double *thr, double *rs_next, int *nactive,
                         int *nactive_clear, int *iters, __nv_bfloat16 *hi, __nv_bfloat16 *lo,
                         cudaStream_t s);
template <typename T>
int launch_cg_direction(T *P, const T *R, int64_t ld, int64_t n, int64_t p, const double *rs,
                        const double *rs_next, const double *thr, __nv_bfloat16 *hi,
                        __nv_bfloat16 *lo, cudaStream_t s);

// adjoint_kernels.cu
int launch_pi_gamma(const double *H, const double *dH, const double *dc, const double *c, int k,
                    int64_t p, double *Pi, cudaStream_t s);
int launch_adj_init(const double *dH, const double *h, int k, int64_t p, double *gamma, double *coef,
                    cudaStream_t s);
int launch_adj_reortho_coef(const double *h, const double *dH, int k, int64_t p, int idx, int ncols,
                            double *coef, cudaStream_t s);
int launch_adj_step_coef(const double *H, const double *Pi, const double *g, const double *gamma,
                         int k, int64_t p, int idx, double *Gamma, double *coefG, double *bp,
                         double *scal, double *beta, cudaStream_t s);
template <typename T>
int launch_adj_lincomb(const T *U, const T *lam, const T *R, const T *dq, int64_t dq_bstride,
                       const double *scal, int64_t n, int64_t ld, int64_t p, T *out, cudaStream_t s);
int launch_axpy_f64(double a, const double *x, double *y, int64_t m, cudaStream_t s);
int gemm_rule_add(int64_t n_lo, int64_t n_hi, int64_t p_lo, int64_t p_hi, int bn, int split);
int gemm_rules_clear();
template <typename T>
int launch_basis_combine(const T *Q, int64_t k, int64_t ld, int64_t n, int64_t p, const double *coef,
                         T *out, cudaStream_t s);

// tridiag_quadrature.cu
int launch_tridiag_eigh_full(int64_t k, int64_t p, const double *H, double *w, double *S,
                             double *Z, int *status, cudaStream_t s);
int launch_tridiag_quadrature(int64_t k, int64_t p, const double *H, int32_t fun, double param,
                              const double *scale, double *values, double *eigvals,
                              double *first_sq, int *status, cudaStream_t s);
int launch_mean_sem(const double *values, int64_t p, double *mean_sem, cudaStream_t s);

// operators.cu
template <typename T>
int launch_dense_simt(const T *A, int64_t lda, const T *V, int64_t ldv, T *W, int64_t ldw,
                      int64_t n, int64_t p, double shift, cudaStream_t s);
int launch_csr_spmm(const int32_t *row_ptr, const int32_t *col_idx, const float *val, int64_t n,
                    int64_t nnz, const float *V, int64_t ldv, float *W, int64_t ldw, int64_t p,
                    double shift, int *status, cudaStream_t s);
int launch_rbf_build(const float *x, int64_t n, int dim, double s2, double ell, int precision,
                     int dlogell, void *a, void *a_lo, int64_t lda, cudaStream_t s);
int launch_split_bf16(const float *a, int64_t rows, int64_t cols, int64_t lda, __nv_bfloat16 *hi,
                      __nv_bfloat16 *lo, int64_t ld_out, cudaStream_t s);

// dense_tcgen05.cu: 2-D tensor map without swizzle (elements of `elem_bytes`
// = 4 or 8, `cols` contiguous, `rows` rows `ld` elements apart, box
// box_cols x box_rows, zero fill out of bounds); false if encoding failed.
bool make_plain_tensor_map_2d(void *map128, int elem_bytes, const void *base, int64_t cols,
                              int64_t rows, int64_t ld, uint32_t box_cols, uint32_t box_rows);

// dense_tcgen05.cu: W = A V with A in bf16 (hi, optionally lo) and the panel
// given as bf16 hi (and lo) copies; fp32 accumulate; W fp32 + shift * Vf.
int launch_dense_tcgen05(const __nv_bfloat16 *A_hi, const __nv_bfloat16 *A_lo, int64_t lda,
                         const __nv_bfloat16 *V_hi, const __nv_bfloat16 *V_lo, int64_t ldvb,
                         const float *Vf, int64_t ldvf, float *W, int64_t ldw, int64_t n,
                         int64_t p, double shift, int *status, cudaStream_t s);
bool tcgen05_supported_shape(int64_t n, int64_t p);

// wait_selftest.cu: a bounded wait on an mbarrier nothing arrives on
int launch_wait_selftest(uint64_t limit_ns, int *status, unsigned long long *times, cudaStream_t s);

}  // namespace mfg
