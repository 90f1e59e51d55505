// C entry points (include/matfree_gb300.h) and the batched Arnoldi driver.
//
// The driver issues, per Krylov step j, on the caller's stream:
//   operator apply  W = A q_j            (tcgen05 GEMM / CUDA-core GEMM / SpMM / callback)
//   projection      H[:, 0..j][j] = Q^T W          (first Gram-Schmidt pass)
//   update          W -= Q H[:, j]
//   projection      h2 = Q^T W                      (second pass, reortho = full)
//   update + norm   W -= Q h2, beta = ||W||, H[j+1][j] = beta
//   normalise       q_{j+1} = W / beta  (+ bf16 hi/lo copies for the tensor cores)
// mirroring matfree/decomp.py:454-477 step by step, batched over the probes.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace mfg {

static thread_local char g_last_error[512] = "";

void record_error(const char *where, int line, const char *what) {
  const char *base = where;
  for (const char *q = where; *q; ++q)
    if (*q == '/') base = q + 1;
  snprintf(g_last_error, sizeof(g_last_error), "%s:%d: %s", base, line, what ? what : "");
}

// ---------------------------------------------------------------------------
// Launch accounting: every kernel the driver issues is counted per class; when
// timing is on, a pair of CUDA events brackets each launch on its stream and
// the launch's algorithmic bytes and flops are recorded with it.  Process-wide
// and meant for benchmarks (one driver thread at a time).
// ---------------------------------------------------------------------------

struct ProfRec {
  int cls;
  size_t e0, e1;
  double bytes, flops;
};

struct Profiler {
  std::mutex mu;
  bool timing = false;
  std::vector<cudaEvent_t> pool;
  size_t next = 0;
  std::vector<ProfRec> recs;
  int64_t launches[MFG_PROF_CLASSES] = {0};
};

static Profiler &prof() {
  static Profiler p;
  return p;
}

static size_t prof_begin(cudaStream_t s) {
  Profiler &P = prof();
  if (!P.timing) return (size_t)-1;
  std::lock_guard<std::mutex> lk(P.mu);
  while (P.pool.size() < P.next + 2) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return (size_t)-1;
    P.pool.push_back(e);
  }
  const size_t e0 = P.next;
  P.next += 2;
  cudaEventRecord(P.pool[e0], s);
  return e0;
}

static void prof_end(size_t e0, int cls, double bytes, double flops, cudaStream_t s) {
  Profiler &P = prof();
  std::lock_guard<std::mutex> lk(P.mu);
  P.launches[cls] += 1;
  if (e0 == (size_t)-1) return;
  cudaEventRecord(P.pool[e0 + 1], s);
  P.recs.push_back(ProfRec{cls, e0, e0 + 1, bytes, flops});
}

#define MFG_LAUNCH(cls, bytes, flops, call)        \
  do {                                             \
    const size_t _e = prof_begin(s);               \
    const int _st = (call);                        \
    prof_end(_e, (cls), (bytes), (flops), s);      \
    if (_st != MFG_OK) return _st;                 \
  } while (0)

struct WsLayout {
  size_t w, panel, norm, len0, h2, partials, counters, status, hi, lo, q, h, values, eig, fsq;
  // two-sweep Arnoldi: qt (float panel), X2 (p (2k + 1)), dots (p 3), nu (p),
  // finish coefficients (p 4), full coefficients Hh (p (k + 1) k)
  size_t vt, x2, dots, nu, cf, hh;
  size_t total;
};

static int elem_size_for(const mfg_operator *op) {
  return op->precision == MFG_PREC_FP64 ? 8 : 4;
}

// The two-sweep step covers float bases of 2 <= k <= kTwoSweepMaxK vectors.
static bool two_sweep_applies(const mfg_operator *op, int64_t k) {
  return op->precision != MFG_PREC_FP64 && k >= 2 && k <= kTwoSweepMaxK;
}

static bool uses_bf16(const mfg_operator *op) {
  return op->kind == MFG_OP_DENSE &&
         (op->precision == MFG_PREC_BF16 || op->precision == MFG_PREC_BF16X3);
}

// The device status word comes first, so that mfg_workspace_status can find
// it without the problem sizes.
static WsLayout layout(const mfg_operator *op, int64_t k, int64_t p, int64_t ld, bool two = false) {
  WsLayout L{};
  const size_t es = (size_t)elem_size_for(op);
  // the fused update+projection uses the smallest chunks (256 rows)
  const int64_t nch = es == 8 ? max_fused_chunks<double>(op->n) : max_fused_chunks<float>(op->n);
  const int64_t kk = k > 0 ? k : 1;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  L.status = take(16);
  L.w = take((size_t)p * ld * es);
  L.panel = take(op->kind == MFG_OP_CALLBACK ? (size_t)p * ld * es : 0);
  L.norm = take((size_t)p * 8);
  L.len0 = take((size_t)p * 8);
  L.h2 = take((size_t)p * kk * 8);
  // partial sums per probe and CTA: k + 1 values, 2 (8 ceil(k / 8)) + 1 for
  // the two-vector projections
  L.partials = take((size_t)p * nch * (two ? 2 * kk + 64 : kk + 1) * 8);
  L.counters = take((size_t)p * 4);
  L.hi = take(uses_bf16(op) ? (size_t)p * ld * 2 : 0);
  L.lo = take(uses_bf16(op) && op->precision == MFG_PREC_BF16X3 ? (size_t)p * ld * 2 : 0);
  L.q = take((size_t)p * kk * ld * es);
  L.h = take((size_t)p * kk * kk * 8);
  L.values = take((size_t)p * 8);
  L.eig = take((size_t)p * kk * 8);
  L.fsq = take((size_t)p * kk * 8);
  if (two) {
    L.vt = take((size_t)p * ld * es);
    L.x2 = take((size_t)p * (2 * kk + 1) * 8);
    L.dots = take((size_t)p * 3 * 8);
    L.nu = take((size_t)p * 8);
    L.cf = take((size_t)p * 4 * 8);
    L.hh = take((size_t)p * (kk + 1) * kk * 8);
  }
  L.total = off + 256;  // slack for aligning the caller's base pointer
  return L;
}

static bool aligned16(const void *ptr) { return ((uintptr_t)ptr & 15u) == 0; }

static int check_op(const mfg_operator *op) {
  if (!op || op->n <= 0) return MFG_ERR_BAD_ARG;
  switch (op->kind) {
    case MFG_OP_DENSE:
      if (!op->a || op->lda < op->n || op->lda % 8 != 0 || !aligned16(op->a)) return MFG_ERR_BAD_ARG;
      if (op->precision == MFG_PREC_BF16X3 && (!op->a_lo || !aligned16(op->a_lo))) return MFG_ERR_BAD_ARG;
      if (op->precision < MFG_PREC_FP32 || op->precision > MFG_PREC_FP64) return MFG_ERR_BAD_ARG;
      return MFG_OK;
    case MFG_OP_CSR:
      if (!op->row_ptr || (op->nnz > 0 && (!op->col_idx || !op->values))) return MFG_ERR_BAD_ARG;
      if (op->precision != MFG_PREC_FP32) return MFG_ERR_UNSUPPORTED;
      return MFG_OK;
    case MFG_OP_CALLBACK:
      if (!op->apply) return MFG_ERR_BAD_ARG;
      if (op->precision != MFG_PREC_FP32 && op->precision != MFG_PREC_FP64) return MFG_ERR_BAD_ARG;
      return MFG_OK;
    default:
      return MFG_ERR_BAD_ARG;
  }
}

static char *ws_base(void *workspace) {
  return reinterpret_cast<char *>(align_up((size_t)workspace, 256));
}

// W (ld) = A V (ldv); vhi/vlo are the bf16 copies of V (ldvb) for the
// tensor-core precisions, panel a contiguous scratch panel for callbacks.
template <typename T>
static int apply_op(const mfg_operator *op, const T *V, int64_t ldv, T *W, int64_t ldw, int64_t p,
                    const __nv_bfloat16 *vhi, const __nv_bfloat16 *vlo, int64_t ldvb, T *panel,
                    int *status, cudaStream_t s) {
  const int64_t n = op->n;
  switch (op->kind) {
    case MFG_OP_DENSE:
      if (op->precision == MFG_PREC_FP32 || op->precision == MFG_PREC_FP64)
        return launch_dense_simt<T>(reinterpret_cast<const T *>(op->a), op->lda, V, ldv, W, ldw, n,
                                    p, op->shift, s);
      if constexpr (sizeof(T) == 4) {
        const __nv_bfloat16 *alo =
            op->precision == MFG_PREC_BF16X3 ? reinterpret_cast<const __nv_bfloat16 *>(op->a_lo) : nullptr;
        return launch_dense_tcgen05(reinterpret_cast<const __nv_bfloat16 *>(op->a), alo, op->lda,
                                    vhi, op->precision == MFG_PREC_BF16X3 ? vlo : nullptr, ldvb,
                                    V, ldv, W, ldw, n, p, op->shift, status, s);
      }
      return MFG_ERR_UNSUPPORTED;
    case MFG_OP_CSR:
      if constexpr (sizeof(T) == 4)
        return launch_csr_spmm(op->row_ptr, op->col_idx, op->values, n, op->nnz, V, ldv, W, ldw, p,
                               op->shift, status, s);
      return MFG_ERR_UNSUPPORTED;
    case MFG_OP_CALLBACK: {
      const T *src = V;
      if (ldv != ldw) {
        MFG_CUDA_TRY(cudaMemcpy2DAsync(panel, ldw * sizeof(T), V, ldv * sizeof(T), n * sizeof(T),
                                       p, cudaMemcpyDeviceToDevice, s));
        src = panel;
      }
      const int rc = op->apply(op->ctx, src, W, n, p, ldw, (void *)s);
      if (rc != 0) {
        record_error(__FILE__, __LINE__, "operator callback returned an error");
        return MFG_ERR_CUDA;
      }
      if (op->shift != 0.0) return MFG_ERR_UNSUPPORTED;  // callbacks fold their own shift
      return MFG_OK;
    }
    default:
      return MFG_ERR_BAD_ARG;
  }
}

// Algorithmic bytes and flops of one operator application to p vectors.
static void apply_cost(const mfg_operator *op, int64_t p, double *bytes, double *flops) {
  const double n = (double)op->n, pp = (double)p;
  const double vec_io = 2.0 * n * pp * 4.0;
  switch (op->kind) {
    case MFG_OP_DENSE: {
      const double mats = op->precision == MFG_PREC_BF16X3 ? 2.0 : 1.0;
      const double es = op->precision == MFG_PREC_FP64 ? 8.0 : (op->precision == MFG_PREC_FP32 ? 4.0 : 2.0);
      *bytes = mats * n * n * es + vec_io * (op->precision == MFG_PREC_FP64 ? 2.0 : 1.0);
      *flops = 2.0 * n * n * pp * (op->precision == MFG_PREC_BF16X3 ? 3.0 : 1.0);
      return;
    }
    case MFG_OP_CSR:
      *bytes = 8.0 * (double)op->nnz + 4.0 * (n + 1.0) + vec_io;
      *flops = 2.0 * (double)op->nnz * pp;
      return;
    default:
      *bytes = vec_io;
      *flops = 0.0;
  }
}

// Full reorthogonalisation in two reads of the basis per step (the second
// projection of step j - 1 is done with the first of step j; see the
// two-sweep notes in lanczos_kernels.cu).  Q row 0 and its bf16 copies are
// in place.  H holds what the reference's H holds; R (optional) is the
// reference's residual w''_{k-1}.  A step whose second projection is large
// raises MFG_ERR_RETRY in the device status word.
template <typename T>
static int run_two_sweep(const mfg_operator *op, int64_t k, int64_t p, int64_t ld, T *Q,
                         double *H, T *R, const WsLayout &L, char *ws, cudaStream_t s) {
  if constexpr (sizeof(T) != 4) {
    return MFG_ERR_UNSUPPORTED;
  } else {
    const int64_t n = op->n;
    const double vecb = (double)n * (double)p * (double)sizeof(T);
    double ab = 0.0, af = 0.0;
    apply_cost(op, p, &ab, &af);
    T *Wb = reinterpret_cast<T *>(ws + L.w);
    T *panel = reinterpret_cast<T *>(ws + L.panel);
    T *Vt = reinterpret_cast<T *>(ws + L.vt);
    double *X2 = reinterpret_cast<double *>(ws + L.x2);
    double *dots = reinterpret_cast<double *>(ws + L.dots);
    double *nu = reinterpret_cast<double *>(ws + L.nu);
    double *cf = reinterpret_cast<double *>(ws + L.cf);
    double *Hh = reinterpret_cast<double *>(ws + L.hh);
    double *partials = reinterpret_cast<double *>(ws + L.partials);
    unsigned *counters = reinterpret_cast<unsigned *>(ws + L.counters);
    int *status = reinterpret_cast<int *>(ws + L.status);
    __nv_bfloat16 *hi = uses_bf16(op) ? reinterpret_cast<__nv_bfloat16 *>(ws + L.hi) : nullptr;
    __nv_bfloat16 *lo = (uses_bf16(op) && op->precision == MFG_PREC_BF16X3)
                            ? reinterpret_cast<__nv_bfloat16 *>(ws + L.lo)
                            : nullptr;
    const double bfb = hi ? (double)n * (double)p * 2.0 * (lo ? 2.0 : 1.0) : 0.0;
    const int64_t qb = k * ld;
    const int64_t koff = k, xs = 2 * k + 1;
    // step 0 as the reference: w = A q_0, h_0 = q_0 . w, u_1 = w - q_0 h_0
    MFG_LAUNCH(MFG_PROF_APPLY, ab, af, apply_op<T>(op, Q, qb, Wb, ld, p, hi, lo, ld, panel, status, s));
    MFG_LAUNCH(MFG_PROF_PROJ, 2.0 * vecb, 2.0 * vecb / sizeof(T),
               launch_proj<T>(Q, qb, ld, 1, Wb, ld, n, p, partials, counters, H, k * k, k, s, status));
    MFG_LAUNCH(MFG_PROF_SUB, 3.0 * vecb, 4.0 * vecb / sizeof(T),
               launch_sub<T>(Q, qb, ld, 1, H, k * k, k, Wb, Wb, ld, n, p, true, true, partials,
                             counters, nu, nullptr, 0, s, status));
    // qt_1 = u_1 / ||u_1|| (and its bf16 copies when another product follows)
    MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb + (k > 1 ? bfb : 0.0), vecb / sizeof(T),
               launch_scale<T>(Wb, ld, n, p, nu, Vt, ld, k > 1 ? hi : nullptr, lo, ld, s));
    for (int64_t j = 1; j < k; ++j) {
      const int nc = (int)j;
      MFG_LAUNCH(MFG_PROF_APPLY, ab, af, apply_op<T>(op, Vt, ld, Wb, ld, p, hi, lo, ld, panel, status, s));
      // [Q^T qt | Q^T w | qt . w] from one read of the basis, in column blocks
      // of at most kTwoSweepPassCols vectors (the later blocks' qt . w goes to
      // a scratch slot: it is the first block's value again)
      for (int c0 = 0; c0 < nc; c0 += kTwoSweepPassCols) {
        const int cn = nc - c0 < kTwoSweepPassCols ? nc - c0 : kTwoSweepPassCols;
        MFG_LAUNCH(MFG_PROF_PROJ, (cn + 2.0) * vecb, 4.0 * cn * vecb / sizeof(T),
                   launch_proj2<T>(Q, qb, ld, c0, cn, Wb, Vt, ld, n, p, partials, counters,
                                   X2 + c0, xs, koff, c0 > 0 ? dots : nullptr, 3, status, s));
      }
      // q_j (unnormalised) = qt - Q Q^T qt into row j, w <- w - Q Q^T w; a
      // later column block continues from the first block's results
      for (int c0 = 0; c0 < nc; c0 += kTwoSweepPassCols) {
        const int cn = nc - c0 < kTwoSweepPassCols ? nc - c0 : kTwoSweepPassCols;
        const T *bin = c0 == 0 ? Vt : Q + j * ld;
        const int64_t bstr = c0 == 0 ? ld : qb;
        MFG_LAUNCH(MFG_PROF_SUBPROJ, (cn + 4.0) * vecb, 4.0 * cn * vecb / sizeof(T),
                   launch_sub2<T>(Q, qb, ld, c0, cn, X2 + c0, xs, koff, Wb, ld, bin, bstr,
                                  Q + j * ld, qb, n, p, partials, counters, dots, status, s));
      }
      MFG_LAUNCH(MFG_PROF_OTHER, 8.0 * p * (3.0 * k + 2.0 * j), 2.0 * p * j * j,
                 launch_twosweep_coef((int)j, (int)k, p, X2, koff, dots, H, Hh, nu, cf, status, s));
      const bool more = j + 1 < k;
      MFG_LAUNCH(MFG_PROF_SCALE, (more || R ? 4.0 : 2.0) * vecb + (more ? bfb : 0.0),
                 3.0 * vecb / sizeof(T),
                 launch_twosweep_finish<T>(Q + j * ld, qb, Wb, ld, n, p, cf,
                                           (more || R) ? Vt : nullptr, more ? hi : nullptr, lo,
                                           ld, s));
    }
    if (R) {
      // the reference's last reorthogonalisation: R = nu_k (qt_k - Q Q^T qt_k)
      const int nc = (int)k;
      MFG_LAUNCH(MFG_PROF_PROJ, (nc + 1.0) * vecb, 2.0 * nc * vecb / sizeof(T),
                 launch_proj<T>(Q, qb, ld, nc, Vt, ld, n, p, partials, counters, X2, xs, 1, s, status));
      MFG_LAUNCH(MFG_PROF_SUB, (nc + 2.0) * vecb, 2.0 * nc * vecb / sizeof(T),
                 launch_sub<T>(Q, qb, ld, nc, X2, xs, 1, Vt, R, ld, n, p, false, true, partials,
                               counters, nullptr, nullptr, 0, s, status));
      MFG_LAUNCH(MFG_PROF_OTHER, 16.0 * p, (double)p, launch_inv(nu, cf, p, s));
      MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb, vecb / sizeof(T),
                 launch_scale<T>(R, ld, n, p, cf, R, ld, nullptr, nullptr, ld, s));
    }
    return MFG_OK;
  }
}

template <typename T>
static int run_hessenberg(const mfg_operator *op, int64_t k, int64_t p, const T *V, int64_t ld,
                          int reortho, T *Q, double *H, T *R, double *init_len_inv,
                          const WsLayout &L, char *ws, cudaStream_t s) {
  const int64_t n = op->n;
  const double vecb = (double)n * (double)p * (double)sizeof(T);  // one panel
  double ab = 0.0, af = 0.0;
  apply_cost(op, p, &ab, &af);
  T *Wb = reinterpret_cast<T *>(ws + L.w);
  T *panel = reinterpret_cast<T *>(ws + L.panel);
  double *norm = reinterpret_cast<double *>(ws + L.norm);
  double *len0 = reinterpret_cast<double *>(ws + L.len0);
  double *h2 = reinterpret_cast<double *>(ws + L.h2);
  double *partials = reinterpret_cast<double *>(ws + L.partials);
  unsigned *counters = reinterpret_cast<unsigned *>(ws + L.counters);
  int *status = reinterpret_cast<int *>(ws + L.status);
  __nv_bfloat16 *hi = uses_bf16(op) ? reinterpret_cast<__nv_bfloat16 *>(ws + L.hi) : nullptr;
  __nv_bfloat16 *lo = (uses_bf16(op) && op->precision == MFG_PREC_BF16X3)
                          ? reinterpret_cast<__nv_bfloat16 *>(ws + L.lo)
                          : nullptr;
  const int64_t qb = k * ld;  // probe stride of the basis

  MFG_CUDA_TRY(cudaMemsetAsync(counters, 0, (size_t)p * 4, s));
  MFG_CUDA_TRY(cudaMemsetAsync(status, 0, 16, s));
  if (k > 0) MFG_CUDA_TRY(cudaMemsetAsync(H, 0, (size_t)p * k * k * 8, s));

  const double bfb = hi ? (double)n * (double)p * 2.0 * (lo ? 2.0 : 1.0) : 0.0;

  // initial length (decomp.py:436) -> 1 / length
  MFG_LAUNCH(MFG_PROF_OTHER, vecb, 2.0 * vecb / sizeof(T),
             launch_sub<T>(nullptr, 0, 0, 0, nullptr, 0, 0, V, nullptr, ld, n, p, true, false,
                           partials, counters, len0, nullptr, 0, s));
  if (init_len_inv) MFG_LAUNCH(MFG_PROF_OTHER, 16.0 * p, (double)p, launch_inv(len0, init_len_inv, p, s));
  if (k == 0) {
    if (R)
      MFG_CUDA_TRY(cudaMemcpy2DAsync(R, ld * sizeof(T), V, ld * sizeof(T), ld * sizeof(T), p,
                                     cudaMemcpyDeviceToDevice, s));
    return MFG_OK;
  }
  MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb + bfb, vecb / sizeof(T),
             launch_scale<T>(V, ld, n, p, len0, Q, qb, hi, lo, ld, s));
  if (reortho == 3) return run_two_sweep<T>(op, k, p, ld, Q, H, R, L, ws, s);

  for (int64_t j = 0; j < k; ++j) {
    const T *qj = Q + j * ld;
    MFG_LAUNCH(MFG_PROF_APPLY, ab, af,
               apply_op<T>(op, qj, qb, Wb, ld, p, hi, lo, ld, panel, status, s));
    const int ncols = (int)(j + 1);
    const double pb = (ncols + 1.0) * vecb, pf = 2.0 * ncols * vecb / sizeof(T);
    const double ub = (ncols + 2.0) * vecb;
    if (reortho == 2) {
      // three-term Lanczos (matfree/decomp.py:215-291): a_j = q_j^T A q_j into
      // H[j][j]; w -= b_{j-1} q_{j-1} + a_j q_j with both coefficients read from
      // row j of H (H[j][j-1] = b_{j-1}, H[j][j] = a_j); b_j = ||w|| into H[j+1][j]
      const bool last3 = (j + 1 == k);
      MFG_LAUNCH(MFG_PROF_PROJ, 2.0 * vecb, 2.0 * vecb / sizeof(T),
                 launch_proj<T>(qj, qb, ld, 1, Wb, ld, n, p, partials, counters, H + j * k + j,
                                k * k, 1, s, status));
      const int nc = j == 0 ? 1 : 2;
      const T *qbase = Q + (j == 0 ? 0 : (j - 1) * ld);
      const double *cf = H + j * k + (j == 0 ? 0 : j - 1);
      MFG_LAUNCH(MFG_PROF_SUB, (nc + 2.0) * vecb, 2.0 * nc * vecb / sizeof(T),
                 launch_sub<T>(qbase, qb, ld, nc, cf, k * k, 1, Wb, Wb, ld, n, p, true, true,
                               partials, counters, norm, last3 ? nullptr : H + (j + 1) * k + j, k * k,
                               s, status));
      if (!last3)
        MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb + bfb, vecb / sizeof(T),
                   launch_scale<T>(Wb, ld, n, p, norm, Q + (j + 1) * ld, qb, hi, lo, ld, s));
      continue;
    }
    // first pass: h = Q^T w into column j of H
    MFG_LAUNCH(MFG_PROF_PROJ, pb, pf,
               launch_proj<T>(Q, qb, ld, ncols, Wb, ld, n, p, partials, counters, H + j, k * k, k, s, status));
    const bool last = (j + 1 == k);
    double *hsub = last ? nullptr : H + (j + 1) * k + j;
    if (reortho && sub_proj_rows_per_thread<T>(ncols) > 0) {
      // w' = w - Q h1 and h2 = Q^T w' from one read of the basis
      MFG_LAUNCH(MFG_PROF_SUBPROJ, (ncols + 2.0) * vecb, 2.0 * pf,
                 launch_sub_proj<T>(Q, qb, ld, ncols, H + j, k * k, k, Wb, ld, n, p, partials,
                                    counters, h2, k, status, s));
      MFG_LAUNCH(MFG_PROF_SUB, ub, pf + 2.0 * vecb / sizeof(T),
                 launch_sub<T>(Q, qb, ld, ncols, h2, k, 1, Wb, Wb, ld, n, p, true, true, partials,
                               counters, norm, hsub, k * k, s, status));
    } else if (reortho) {
      MFG_LAUNCH(MFG_PROF_SUB, ub, pf,
                 launch_sub<T>(Q, qb, ld, ncols, H + j, k * k, k, Wb, Wb, ld, n, p, false, true,
                               partials, counters, norm, nullptr, 0, s, status));
      MFG_LAUNCH(MFG_PROF_PROJ, pb, pf,
                 launch_proj<T>(Q, qb, ld, ncols, Wb, ld, n, p, partials, counters, h2, k, 1, s, status));
      MFG_LAUNCH(MFG_PROF_SUB, ub, pf + 2.0 * vecb / sizeof(T),
                 launch_sub<T>(Q, qb, ld, ncols, h2, k, 1, Wb, Wb, ld, n, p, true, true, partials,
                               counters, norm, hsub, k * k, s, status));
    } else {
      MFG_LAUNCH(MFG_PROF_SUB, ub, pf + 2.0 * vecb / sizeof(T),
                 launch_sub<T>(Q, qb, ld, ncols, H + j, k * k, k, Wb, Wb, ld, n, p, true, true,
                               partials, counters, norm, hsub, k * k, s, status));
    }
    if (!last)
      MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb + bfb, vecb / sizeof(T),
                 launch_scale<T>(Wb, ld, n, p, norm, Q + (j + 1) * ld, qb, hi, lo, ld, s));
  }
  if (R)
    MFG_CUDA_TRY(cudaMemcpy2DAsync(R, ld * sizeof(T), Wb, ld * sizeof(T), ld * sizeof(T), p,
                                   cudaMemcpyDeviceToDevice, s));
  return MFG_OK;
}

// ---------------------------------------------------------------------------
// Batched Hessenberg adjoint (reverse Arnoldi), matfree/decomp.py:480-600.
// ---------------------------------------------------------------------------

struct AdjLayout {
  size_t lam, lam2, U, panel, h, g, coef, bp, gamma, scal, beta, Gamma, Pi, M, inv, partials,
      counters, status, hi, lo, total;
};

static AdjLayout adj_layout(const mfg_operator *op, int64_t k, int64_t p, int64_t ld) {
  AdjLayout L{};
  const size_t es = (size_t)elem_size_for(op);
  const int64_t nch = es == 8 ? max_fused_chunks<double>(op->n) : max_fused_chunks<float>(op->n);
  const int64_t kk = k > 0 ? k : 1;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  L.lam = take((size_t)p * ld * es);
  L.lam2 = take((size_t)p * ld * es);
  L.U = take((size_t)p * ld * es);
  L.panel = take(op->kind == MFG_OP_CALLBACK ? (size_t)p * ld * es : 0);
  L.h = take((size_t)p * kk * 8);
  L.g = take((size_t)p * kk * 8);
  L.coef = take((size_t)p * kk * 8);
  L.bp = take((size_t)p * kk * 8);
  L.gamma = take((size_t)p * kk * 8);
  L.scal = take((size_t)p * 3 * 8);
  L.beta = take((size_t)p * 8);
  L.Gamma = take((size_t)p * kk * kk * 8);
  L.Pi = take((size_t)p * kk * kk * 8);
  L.M = take((size_t)p * kk * kk * 8);
  L.inv = take((size_t)p * 8);
  L.partials = take((size_t)p * nch * (kk + 1) * 8);
  L.counters = take((size_t)p * 4);
  L.status = take(16);
  L.hi = take(uses_bf16(op) ? (size_t)p * ld * 2 : 0);
  L.lo = take(uses_bf16(op) && op->precision == MFG_PREC_BF16X3 ? (size_t)p * ld * 2 : 0);
  L.total = off + 256;
  return L;
}

template <typename T>
static int run_adjoint(const mfg_operator *op, int64_t k, int64_t p, int64_t ld, const T *Q,
                       const double *H, const T *R, const double *c, const T *dQ, const double *dH,
                       const T *dr, const double *dc, T *Lam, T *dv, const AdjLayout &L, char *ws,
                       cudaStream_t s) {
  const int64_t n = op->n;
  const int64_t qb = k * ld;
  T *lam = reinterpret_cast<T *>(ws + L.lam);
  T *lam2 = reinterpret_cast<T *>(ws + L.lam2);
  T *U = reinterpret_cast<T *>(ws + L.U);
  T *panel = reinterpret_cast<T *>(ws + L.panel);
  double *h = reinterpret_cast<double *>(ws + L.h);
  double *g = reinterpret_cast<double *>(ws + L.g);
  double *coef = reinterpret_cast<double *>(ws + L.coef);
  double *bp = reinterpret_cast<double *>(ws + L.bp);
  double *gamma = reinterpret_cast<double *>(ws + L.gamma);
  double *scal = reinterpret_cast<double *>(ws + L.scal);
  double *beta = reinterpret_cast<double *>(ws + L.beta);
  double *Gamma = reinterpret_cast<double *>(ws + L.Gamma);
  double *Pi = reinterpret_cast<double *>(ws + L.Pi);
  double *inv = reinterpret_cast<double *>(ws + L.inv);
  double *partials = reinterpret_cast<double *>(ws + L.partials);
  unsigned *counters = reinterpret_cast<unsigned *>(ws + L.counters);
  int *status = reinterpret_cast<int *>(ws + L.status);
  __nv_bfloat16 *hi = uses_bf16(op) ? reinterpret_cast<__nv_bfloat16 *>(ws + L.hi) : nullptr;
  __nv_bfloat16 *lo = (uses_bf16(op) && op->precision == MFG_PREC_BF16X3)
                          ? reinterpret_cast<__nv_bfloat16 *>(ws + L.lo)
                          : nullptr;
  const double vecb = (double)n * (double)p * (double)sizeof(T);
  double ab = 0.0, af = 0.0;
  apply_cost(op, p, &ab, &af);

  MFG_CUDA_TRY(cudaMemsetAsync(counters, 0, (size_t)p * 4, s));
  MFG_CUDA_TRY(cudaMemsetAsync(status, 0, 16, s));
  MFG_CUDA_TRY(cudaMemsetAsync(Gamma, 0, (size_t)p * k * k * 8, s));
  MFG_CUDA_TRY(cudaMemsetAsync(lam, 0, (size_t)p * ld * sizeof(T), s));
  MFG_LAUNCH(MFG_PROF_OTHER, 24.0 * p * k * k, 2.0 * p * k * k * k,
             launch_pi_gamma(H, dH, dc, c, (int)k, p, Pi, s));
  if (dQ) {
    // Pi_gamma -= dQ^T Q   (decomp.py:506): row i of M is Q^T dq_i, one sweep per column of dQ
    double *M = reinterpret_cast<double *>(ws + L.M);
    for (int64_t i = 0; i < k; ++i)
      MFG_LAUNCH(MFG_PROF_PROJ, (k + 1.0) * vecb, 2.0 * k * vecb / sizeof(T),
                 launch_proj<T>(Q, qb, ld, (int)k, dQ + i * ld, qb, n, p, partials, counters, M + i * k,
                                k * k, 1, s, status));
    MFG_LAUNCH(MFG_PROF_OTHER, 24.0 * p * k * k, (double)p * k * k,
               launch_axpy_f64(-1.0, M, Pi, p * k * k, s));
  }
  // gamma = dH e_K - Q^T dr ;  lambda = dr + Q gamma   (decomp.py:498-499)
  if (dr) {
    MFG_LAUNCH(MFG_PROF_PROJ, (k + 1.0) * vecb, 2.0 * k * vecb / sizeof(T),
               launch_proj<T>(Q, qb, ld, (int)k, dr, ld, n, p, partials, counters, h, k, 1, s, status));
    MFG_CUDA_TRY(cudaMemcpy2DAsync(lam, ld * sizeof(T), dr, ld * sizeof(T), ld * sizeof(T), p,
                                   cudaMemcpyDeviceToDevice, s));
  }
  MFG_LAUNCH(MFG_PROF_OTHER, 16.0 * p * k, (double)p * k,
             launch_adj_init(dH, dr ? h : nullptr, (int)k, p, gamma, coef, s));
  MFG_LAUNCH(MFG_PROF_SUB, (k + 2.0) * vecb, 2.0 * k * vecb / sizeof(T),
             launch_sub<T>(Q, qb, ld, (int)k, coef, k, 1, lam, lam, ld, n, p, false, true, partials,
                           counters, nullptr, nullptr, 0, s, status));

  for (int64_t idx = k - 1; idx >= 0; --idx) {
    const int ncr = (int)(idx + 2 < k ? idx + 2 : k);
    // masked re-projection: lambda -= Q_m (Q_m^T lambda - dH[:, idx]_m)   (decomp.py:576-584)
    MFG_LAUNCH(MFG_PROF_PROJ, (ncr + 1.0) * vecb, 2.0 * ncr * vecb / sizeof(T),
               launch_proj<T>(Q, qb, ld, ncr, lam, ld, n, p, partials, counters, h, k, 1, s, status));
    MFG_LAUNCH(MFG_PROF_OTHER, 16.0 * p * ncr, (double)p * ncr,
               launch_adj_reortho_coef(h, dH, (int)k, p, (int)idx, ncr, coef, s));
    MFG_LAUNCH(MFG_PROF_SUB, (ncr + 2.0) * vecb, 2.0 * ncr * vecb / sizeof(T),
               launch_sub<T>(Q, qb, ld, ncr, coef, k, 1, lam, lam, ld, n, p, false, true, partials,
                             counters, nullptr, nullptr, 0, s, status));
    // U = A^T lambda (= A lambda: tridiag_sym's operators are symmetric)   (decomp.py:587-589)
    if (hi) MFG_TRY(launch_split_bf16((const float *)lam, p, n, ld, hi, lo, ld, s));
    MFG_LAUNCH(MFG_PROF_APPLY, ab, af, apply_op<T>(op, lam, ld, U, ld, p, hi, lo, ld, panel, status, s));
    // Gamma row idx, (Gamma + Gamma^T)[idx, :], beta_plus row   (decomp.py:592-599)
    MFG_LAUNCH(MFG_PROF_PROJ, (idx + 2.0) * vecb, 2.0 * (idx + 1.0) * vecb / sizeof(T),
               launch_proj<T>(Q, qb, ld, (int)(idx + 1), U, ld, n, p, partials, counters, g, k, 1, s, status));
    MFG_LAUNCH(MFG_PROF_OTHER, 40.0 * p * k, 4.0 * p * k,
               launch_adj_step_coef(H, Pi, g, gamma, (int)k, p, (int)idx, Gamma, coef, bp, scal,
                                    beta, s));
    MFG_CUDA_TRY(cudaMemcpy2DAsync(Lam + idx * ld, qb * sizeof(T), lam, ld * sizeof(T),
                                   ld * sizeof(T), p, cudaMemcpyDeviceToDevice, s));
    // lambda = (gamma_idx r + Q G - alpha lambda + U - Lambda beta_plus) / beta_minus
    // Pi_xi row idx = dq_idx + gamma_idx r   (decomp.py:505)
    MFG_LAUNCH(MFG_PROF_SCALE, (dQ ? 5.0 : 4.0) * vecb, (dQ ? 4.0 : 3.0) * vecb / sizeof(T),
               launch_adj_lincomb<T>(U, lam, R, dQ ? dQ + idx * ld : nullptr, qb, scal, n, ld, p, lam2,
                                     s));
    MFG_LAUNCH(MFG_PROF_SUB, (k + 2.0) * vecb, 2.0 * k * vecb / sizeof(T),
               launch_sub<T>(Q, qb, ld, (int)k, coef, k, 1, lam2, lam2, ld, n, p, false, true,
                             partials, counters, nullptr, nullptr, 0, s, status));
    if (idx + 1 < k) {
      const int nb = (int)(k - idx - 1);
      MFG_LAUNCH(MFG_PROF_SUB, (nb + 2.0) * vecb, 2.0 * nb * vecb / sizeof(T),
                 launch_sub<T>(Lam + (idx + 1) * ld, qb, ld, nb, bp + idx + 1, k, 1, lam2, lam2, ld,
                               n, p, false, true, partials, counters, nullptr, nullptr, 0, s, status));
    }
    MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb, vecb / sizeof(T),
               launch_scale<T>(lam2, ld, n, p, beta, lam, ld, nullptr, nullptr, 0, s));
  }
  // dv = lambda c   (decomp.py:541)
  MFG_LAUNCH(MFG_PROF_OTHER, 16.0 * p, (double)p, launch_inv(c, inv, p, s));
  MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb, vecb / sizeof(T),
             launch_scale<T>(lam, ld, n, p, inv, dv, ld, nullptr, nullptr, 0, s));
  return MFG_OK;
}

__global__ void square_kernel(const double *x, double *y, int64_t p) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b < p) y[b] = x[b] * x[b];
}

static int launch_square(const double *x, double *y, int64_t p, cudaStream_t s) {
  square_kernel<<<(unsigned)ceil_div(p, 128), 128, 0, s>>>(x, y, p);
  return MFG_LAUNCH_STATUS();
}

}  // namespace mfg

using namespace mfg;

// ---------------------------------------------------------------------------
// Golub-Kahan bidiagonalisation with full reorthogonalisation
// (matfree/decomp.py:608-750), batched over the probe rows of a panel, and
// the product quadrature e1^T f(B^T B) e1 (matfree/funm.py:246-303)
// ---------------------------------------------------------------------------

struct BidiagLayout {
  WsLayout base;  // working panel, norms, projections, partials, bf16 copies
  size_t u, v, alphas, betas, gram, values, total;
};

static BidiagLayout bidiag_layout(const mfg_operator *A, const mfg_operator *At, int64_t k,
                                  int64_t p, int64_t ld) {
  BidiagLayout L{};
  // bf16 copies of the panel when either operator runs on the tensor cores
  const mfg_operator *big = uses_bf16(At) && !uses_bf16(A) ? At : A;
  if (uses_bf16(At) && At->precision == MFG_PREC_BF16X3) big = At;
  L.base = layout(big, k, p, ld);
  const size_t es = (size_t)elem_size_for(A);
  const int64_t kk = k > 0 ? k : 1;
  size_t off = L.base.total;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  L.u = take((size_t)p * kk * ld * es);
  L.v = take((size_t)p * kk * ld * es);
  L.alphas = take((size_t)p * kk * 8);
  L.betas = take((size_t)p * kk * 8);
  L.gram = take((size_t)p * kk * kk * 8);
  L.values = take((size_t)p * 8);
  L.total = off + 256;
  return L;
}

// H_b = B_b^T B_b for the upper bidiagonal B_b (alphas on the diagonal,
// betas[1:] above it): diagonal a_i^2 + b_i^2 (b_0 = 0), off-diagonal a_i b_{i+1}
__global__ void bidiag_gram_kernel(const double *__restrict__ alphas, const double *__restrict__ betas,
                                   int64_t k, int64_t p, double *__restrict__ H) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= p * k) return;
  const int64_t b = t / k, i = t - b * k;
  const double a = alphas[b * k + i];
  const double bi = i > 0 ? betas[b * k + i] : 0.0;
  double *Hb = H + b * k * k;
  Hb[i * k + i] = a * a + bi * bi;
  if (i + 1 < k) {
    const double o = a * betas[b * k + i + 1];
    Hb[i * k + i + 1] = o;
    Hb[(i + 1) * k + i] = o;
  }
}

template <typename T>
static int run_bidiag(const mfg_operator *A, const mfg_operator *At, int64_t k, int64_t p,
                      const T *V0, int64_t ld, T *U, T *Vb, double *alphas, double *betas, T *R,
                      double *init_len_inv, const BidiagLayout &BL, char *ws, cudaStream_t s) {
  const WsLayout &L = BL.base;
  const int64_t n = A->n;
  const int64_t qb = k * ld;  // probe stride of the bases
  const double vecb = (double)n * (double)p * (double)sizeof(T);
  double ab = 0.0, af = 0.0, tb = 0.0, tf = 0.0;
  apply_cost(A, p, &ab, &af);
  apply_cost(At, p, &tb, &tf);
  T *Wb = reinterpret_cast<T *>(ws + L.w);
  T *panel = reinterpret_cast<T *>(ws + L.panel);
  double *norm = reinterpret_cast<double *>(ws + L.norm);
  double *len0 = reinterpret_cast<double *>(ws + L.len0);
  double *h1 = reinterpret_cast<double *>(ws + L.h);
  double *h2 = reinterpret_cast<double *>(ws + L.h2);
  double *partials = reinterpret_cast<double *>(ws + L.partials);
  unsigned *counters = reinterpret_cast<unsigned *>(ws + L.counters);
  int *status = reinterpret_cast<int *>(ws + L.status);
  const bool bf = uses_bf16(A) || uses_bf16(At);
  const bool bflo = (uses_bf16(A) && A->precision == MFG_PREC_BF16X3) ||
                    (uses_bf16(At) && At->precision == MFG_PREC_BF16X3);
  __nv_bfloat16 *hi = bf ? reinterpret_cast<__nv_bfloat16 *>(ws + L.hi) : nullptr;
  __nv_bfloat16 *lo = bflo ? reinterpret_cast<__nv_bfloat16 *>(ws + L.lo) : nullptr;
  const __nv_bfloat16 *hiA = uses_bf16(A) ? hi : nullptr;
  const __nv_bfloat16 *loA = uses_bf16(A) && A->precision == MFG_PREC_BF16X3 ? lo : nullptr;
  const __nv_bfloat16 *hiT = uses_bf16(At) ? hi : nullptr;
  const __nv_bfloat16 *loT = uses_bf16(At) && At->precision == MFG_PREC_BF16X3 ? lo : nullptr;

  MFG_CUDA_TRY(cudaMemsetAsync(counters, 0, (size_t)p * 4, s));
  MFG_CUDA_TRY(cudaMemsetAsync(status, 0, 16, s));
  if (k > 0) {
    MFG_CUDA_TRY(cudaMemsetAsync(alphas, 0, (size_t)p * k * 8, s));
    MFG_CUDA_TRY(cudaMemsetAsync(betas, 0, (size_t)p * k * 8, s));
  }
  // ||v0|| (decomp.py:683) -> 1 / length; v_0 = v0 / ||v0||
  MFG_LAUNCH(MFG_PROF_OTHER, vecb, 2.0 * vecb / sizeof(T),
             launch_sub<T>(nullptr, 0, 0, 0, nullptr, 0, 0, V0, nullptr, ld, n, p, true, false,
                           partials, counters, len0, nullptr, 0, s));
  if (init_len_inv) MFG_LAUNCH(MFG_PROF_OTHER, 16.0 * p, (double)p, launch_inv(len0, init_len_inv, p, s));
  if (k == 0) {
    if (R) MFG_CUDA_TRY(cudaMemsetAsync(R, 0, (size_t)p * ld * sizeof(T), s));
    return MFG_OK;
  }
  MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb, vecb / sizeof(T),
             launch_scale<T>(V0, ld, n, p, len0, Vb, qb, hi, lo, ld, s));

  // CGS2 of the working panel against `ncols` basis rows, then ||w|| into
  // norm (and out2[b * o2s] when given), as in decomp.py:703-719
  auto cgs2 = [&](const T *Q, int ncols, double *out2, int64_t o2s) -> int {
    if (ncols == 0)
      return launch_sub<T>(nullptr, 0, 0, 0, nullptr, 0, 0, Wb, Wb, ld, n, p, true, false, partials,
                           counters, norm, out2, o2s, s, status);
    const double pb = (ncols + 1.0) * vecb, pf = 2.0 * ncols * vecb / sizeof(T);
    const double ub = (ncols + 2.0) * vecb;
    MFG_LAUNCH(MFG_PROF_PROJ, pb, pf,
               launch_proj<T>(Q, qb, ld, ncols, Wb, ld, n, p, partials, counters, h1, k, 1, s, status));
    if (sub_proj_rows_per_thread<T>(ncols) > 0) {
      MFG_LAUNCH(MFG_PROF_SUBPROJ, (ncols + 2.0) * vecb, 2.0 * pf,
                 launch_sub_proj<T>(Q, qb, ld, ncols, h1, k, 1, Wb, ld, n, p, partials, counters, h2,
                                    k, status, s));
    } else {
      MFG_LAUNCH(MFG_PROF_SUB, ub, pf,
                 launch_sub<T>(Q, qb, ld, ncols, h1, k, 1, Wb, Wb, ld, n, p, false, true, partials,
                               counters, norm, nullptr, 0, s, status));
      MFG_LAUNCH(MFG_PROF_PROJ, pb, pf,
                 launch_proj<T>(Q, qb, ld, ncols, Wb, ld, n, p, partials, counters, h2, k, 1, s,
                                status));
    }
    MFG_LAUNCH(MFG_PROF_SUB, ub, pf + 2.0 * vecb / sizeof(T),
               launch_sub<T>(Q, qb, ld, ncols, h2, k, 1, Wb, Wb, ld, n, p, true, true, partials,
                             counters, norm, out2, o2s, s, status));
    return MFG_OK;
  };

  for (int64_t i = 0; i < k; ++i) {
    // left vector: u_i = (A v_i - beta_i u_{i-1}) reorthogonalised, / alpha_i
    MFG_LAUNCH(MFG_PROF_APPLY, ab, af,
               apply_op<T>(A, Vb + i * ld, qb, Wb, ld, p, hiA, loA, ld, panel, status, s));
    if (i > 0)
      MFG_LAUNCH(MFG_PROF_SUB, 3.0 * vecb, 2.0 * vecb / sizeof(T),
                 launch_sub<T>(U + (i - 1) * ld, qb, ld, 1, betas + i, k, 1, Wb, Wb, ld, n, p, false,
                               true, partials, counters, norm, nullptr, 0, s, status));
    MFG_TRY(cgs2(U, (int)i, alphas + i, k));
    MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb, vecb / sizeof(T),
               launch_scale<T>(Wb, ld, n, p, norm, U + i * ld, qb, hi, lo, ld, s));
    // right vector: v_{i+1} = (A^T u_i - alpha_i v_i) reorthogonalised, / beta_{i+1}
    MFG_LAUNCH(MFG_PROF_APPLY, tb, tf,
               apply_op<T>(At, U + i * ld, qb, Wb, ld, p, hiT, loT, ld, panel, status, s));
    MFG_LAUNCH(MFG_PROF_SUB, 3.0 * vecb, 2.0 * vecb / sizeof(T),
               launch_sub<T>(Vb + i * ld, qb, ld, 1, alphas + i, k, 1, Wb, Wb, ld, n, p, false, true,
                             partials, counters, norm, nullptr, 0, s, status));
    const bool last = i + 1 == k;
    MFG_TRY(cgs2(Vb, (int)(i + 1), last ? nullptr : betas + i + 1, k));
    if (!last)
      MFG_LAUNCH(MFG_PROF_SCALE, 2.0 * vecb, vecb / sizeof(T),
                 launch_scale<T>(Wb, ld, n, p, norm, Vb + (i + 1) * ld, qb, hi, lo, ld, s));
  }
  // residual = beta_k v_k = the last reorthogonalised right vector (decomp.py:736)
  if (R)
    MFG_CUDA_TRY(cudaMemcpy2DAsync(R, ld * sizeof(T), Wb, ld * sizeof(T), ld * sizeof(T), p,
                                   cudaMemcpyDeviceToDevice, s));
  return MFG_OK;
}

// ---------------------------------------------------------------------------
// Conjugate gradients (jax.scipy.sparse.linalg.cg with x0 = 0 and no
// preconditioner, one independent solve per probe row of the panel)
// ---------------------------------------------------------------------------

constexpr int64_t kCgCheckEvery = 8;  // iterations between host convergence tests

struct CgLayout {
  size_t r, p, w, hi, lo, rs0, rs1, pap, thr, partials, counters, nactive, status, iters, total;
};

static CgLayout cg_layout(const mfg_operator *op, int64_t p, int64_t ld) {
  CgLayout L{};
  const size_t es = (size_t)elem_size_for(op);
  const int64_t nch = es == 8 ? max_fused_chunks<double>(op->n) : max_fused_chunks<float>(op->n);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off = align_up(off + bytes, 256);
    return o;
  };
  L.r = take((size_t)p * ld * es);
  L.p = take((size_t)p * ld * es);
  L.w = take((size_t)p * ld * es);
  L.hi = take(uses_bf16(op) ? (size_t)p * ld * 2 : 0);
  L.lo = take(uses_bf16(op) && op->precision == MFG_PREC_BF16X3 ? (size_t)p * ld * 2 : 0);
  L.rs0 = take((size_t)p * 8);
  L.rs1 = take((size_t)p * 8);
  L.pap = take((size_t)p * 8);
  L.thr = take((size_t)p * 8);
  L.partials = take((size_t)p * nch * 8);
  L.counters = take((size_t)p * 4);
  L.nactive = take(16);
  L.status = take(16);
  L.iters = take((size_t)p * 4);
  L.total = off + 256;
  return L;
}

template <typename T>
static int run_cg(const mfg_operator *op, int64_t p, const T *B, T *X, int64_t ld, double tol,
                  double atol, int64_t maxiter, int32_t *iters_out, const CgLayout &L, char *ws,
                  cudaStream_t s) {
  const int64_t n = op->n;
  T *R = reinterpret_cast<T *>(ws + L.r);
  T *P = reinterpret_cast<T *>(ws + L.p);
  T *W = reinterpret_cast<T *>(ws + L.w);
  __nv_bfloat16 *hi = uses_bf16(op) ? reinterpret_cast<__nv_bfloat16 *>(ws + L.hi) : nullptr;
  __nv_bfloat16 *lo = (uses_bf16(op) && op->precision == MFG_PREC_BF16X3)
                          ? reinterpret_cast<__nv_bfloat16 *>(ws + L.lo)
                          : nullptr;
  double *rs[2] = {reinterpret_cast<double *>(ws + L.rs0), reinterpret_cast<double *>(ws + L.rs1)};
  double *pap = reinterpret_cast<double *>(ws + L.pap);
  double *thr = reinterpret_cast<double *>(ws + L.thr);
  double *partials = reinterpret_cast<double *>(ws + L.partials);
  unsigned *counters = reinterpret_cast<unsigned *>(ws + L.counters);
  int *nactive = reinterpret_cast<int *>(ws + L.nactive);
  int *status = reinterpret_cast<int *>(ws + L.status);
  int *iters = iters_out ? iters_out : reinterpret_cast<int *>(ws + L.iters);
  const double vecb = (double)n * (double)p * (double)sizeof(T);
  double ab = 0.0, af = 0.0;
  apply_cost(op, p, &ab, &af);

  MFG_CUDA_TRY(cudaMemsetAsync(counters, 0, (size_t)p * 4, s));
  MFG_CUDA_TRY(cudaMemsetAsync(status, 0, 16, s));
  MFG_CUDA_TRY(cudaMemsetAsync(nactive, 0, 2 * sizeof(int), s));
  MFG_LAUNCH(MFG_PROF_OTHER, 4.0 * vecb, 2.0 * vecb / sizeof(T),
             launch_cg_init<T>(B, X, R, P, ld, n, p, hi, lo, partials, counters, tol * tol,
                               atol * atol, rs[0], thr, iters, s));
  // Iteration it counts the rows that keep running into nactive[it & 1] and
  // zeroes nactive[(it + 1) & 1] for the next one.
  const bool small = n <= kCgSmallMaxN;
  auto iteration = [&](int64_t it) -> int {
    double *rc = rs[it & 1], *rn = rs[(it + 1) & 1];
    int *na = nactive + (it & 1), *na_next = nactive + ((it + 1) & 1);
    MFG_LAUNCH(MFG_PROF_APPLY, ab, af, apply_op<T>(op, P, ld, W, ld, p, hi, lo, ld, nullptr, status, s));
    if (small) {
      MFG_LAUNCH(MFG_PROF_SUB, 7.0 * vecb, 10.0 * vecb / sizeof(T),
                 launch_cg_step_small<T>(X, R, P, W, ld, n, p, rc, thr, rn, na, na_next, iters,
                                         hi, lo, s));
      return MFG_OK;
    }
    MFG_LAUNCH(MFG_PROF_PROJ, 2.0 * vecb, 2.0 * vecb / sizeof(T),
               launch_proj<T>(P, ld, ld, 1, W, ld, n, p, partials, counters, pap, 1, 1, s, status));
    MFG_LAUNCH(MFG_PROF_SUB, 6.0 * vecb, 6.0 * vecb / sizeof(T),
               launch_cg_update<T>(X, R, P, W, ld, n, p, rc, pap, thr, partials, counters, rn,
                                   na, na_next, iters, s));
    MFG_LAUNCH(MFG_PROF_SCALE, 3.0 * vecb, 2.0 * vecb / sizeof(T),
               launch_cg_direction<T>(P, R, ld, n, p, rc, rn, thr, hi, lo, s));
    return MFG_OK;
  };
  // Iterations run in blocks of kCgCheckEvery between convergence tests (a
  // finished row only runs frozen, alpha = 0, iterations until then).  A full
  // block's launches are captured once as a CUDA graph and replayed, which
  // removes the launch gaps between the small kernels of an iteration (the
  // launch counters then count a block's launches once).  Not for callback
  // operators (host code) or while launches are being timed.
  const bool graphs = !prof().timing && op->kind != MFG_OP_CALLBACK;
  cudaGraphExec_t exec = nullptr;
  bool capture_failed = false;
  int rc_loop = MFG_OK;
  for (int64_t it = 0; it < maxiter;) {
    const int64_t blk = maxiter - it < kCgCheckEvery ? maxiter - it : kCgCheckEvery;
    bool done = false;
    if (graphs && !capture_failed && blk == kCgCheckEvery) {
      if (!exec) {
        capture_failed = true;
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
          int st = MFG_OK;
          for (int64_t t = 0; t < blk && st == MFG_OK; ++t) st = iteration(it + t);
          cudaGraph_t g = nullptr;
          const cudaError_t ec = cudaStreamEndCapture(s, &g);
          if (st == MFG_OK && ec == cudaSuccess && g &&
              cudaGraphInstantiate(&exec, g, 0) == cudaSuccess)
            capture_failed = false;
          if (g) cudaGraphDestroy(g);
        }
        (void)cudaGetLastError();  // a failed capture leaves nothing queued: run eagerly
      }
      if (exec && cudaGraphLaunch(exec, s) == cudaSuccess) done = true;
    }
    for (int64_t t = 0; !done && t < blk && rc_loop == MFG_OK; ++t) rc_loop = iteration(it + t);
    if (rc_loop != MFG_OK) break;
    const int *last_count = nactive + ((it + blk - 1) & 1);
    it += blk;
    int host_active = 0;
    if (cudaMemcpyAsync(&host_active, last_count, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      rc_loop = cuda_status(cudaGetLastError(), __FILE__, __LINE__);
      if (rc_loop == MFG_OK) rc_loop = MFG_ERR_CUDA;
      break;
    }
    if (host_active == 0) break;
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (rc_loop != MFG_OK) return rc_loop;
  int host_status = 0;
  MFG_CUDA_TRY(cudaMemcpyAsync(&host_status, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  MFG_CUDA_TRY(cudaStreamSynchronize(s));
  return host_status;
}

extern "C" {

int mfg_version(void) { return 100; }

const char *mfg_last_error(void) { return g_last_error; }

int mfg_profile_enable(int timing) {
  Profiler &P = prof();
  std::lock_guard<std::mutex> lk(P.mu);
  P.timing = timing != 0;
  P.next = 0;
  P.recs.clear();
  for (int c = 0; c < MFG_PROF_CLASSES; ++c) P.launches[c] = 0;
  return MFG_OK;
}

int mfg_profile_read(int32_t nclasses, double *ms, double *bytes, double *flops, int64_t *launches) {
  if (nclasses <= 0 || nclasses > MFG_PROF_CLASSES) return MFG_ERR_BAD_ARG;
  Profiler &P = prof();
  std::lock_guard<std::mutex> lk(P.mu);
  for (int c = 0; c < nclasses; ++c) {
    if (ms) ms[c] = 0.0;
    if (bytes) bytes[c] = 0.0;
    if (flops) flops[c] = 0.0;
    if (launches) launches[c] = P.launches[c];
  }
  for (const ProfRec &r : P.recs) {
    if (r.cls >= nclasses) continue;
    if (cudaEventSynchronize(P.pool[r.e1]) != cudaSuccess) return MFG_ERR_CUDA;
    float t = 0.f;
    if (cudaEventElapsedTime(&t, P.pool[r.e0], P.pool[r.e1]) != cudaSuccess) return MFG_ERR_CUDA;
    if (ms) ms[r.cls] += t;
    if (bytes) bytes[r.cls] += r.bytes;
    if (flops) flops[r.cls] += r.flops;
  }
  return MFG_OK;
}

const char *mfg_status_string(int status) {
  switch (status) {
    case MFG_OK: return "ok";
    case MFG_ERR_BAD_ARG: return "invalid argument";
    case MFG_ERR_RANGE: return "num_matvecs exceeds the acceptable range";
    case MFG_ERR_WORKSPACE: return "workspace too small";
    case MFG_ERR_CUDA: return "CUDA error";
    case MFG_ERR_UNSUPPORTED: return "unsupported operator/precision/shape";
    case MFG_ERR_NO_CONVERGENCE: return "tridiagonal eigensolver did not converge";
    case MFG_ERR_TIMEOUT: return "a bounded device-side wait timed out";
    case MFG_ERR_SCRATCH_LIMIT:
      return "problem exceeds the fixed 32 MiB scratch of the no-allocation entry point";
    case MFG_ERR_RETRY:
      return "two-sweep reorthogonalisation lost accuracy; repeat with the three-sweep form";
    default: return "unknown status";
  }
}

size_t mfg_slq_workspace_bytes(const mfg_operator *op, int64_t k, int64_t p, int64_t ld) {
  if (check_op(op) != MFG_OK || k < 0 || p <= 0 || ld < op->n) return 0;
  return layout(op, k, p, ld).total;
}

static int check_panel(const mfg_operator *op, int64_t p, int64_t ld) {
  if (p <= 0 || p > 65535 || ld < op->n || ld % 8 != 0) return MFG_ERR_BAD_ARG;
  return MFG_OK;
}

int mfg_sampler_signs(const uint32_t key[2], int64_t num, int64_t n, int64_t ld, int32_t dtype,
                      void *out, void *stream) {
  if (!key || !out || n <= 0 || ld < n || ld % 8 != 0 || num < 0 || !aligned16(out))
    return MFG_ERR_BAD_ARG;
  cudaStream_t s = as_stream(stream);
  const double b = (double)num * ld * (dtype == MFG_F64 ? 8.0 : 4.0);
  if (dtype == MFG_F32)
    MFG_LAUNCH(MFG_PROF_OTHER, b, 0.0, launch_sampler<float>(0, key[0], key[1], num, n, ld, (float *)out, s));
  else if (dtype == MFG_F64)
    MFG_LAUNCH(MFG_PROF_OTHER, b, 0.0, launch_sampler<double>(0, key[0], key[1], num, n, ld, (double *)out, s));
  else
    return MFG_ERR_BAD_ARG;
  return MFG_OK;
}

int mfg_sampler_normal(const uint32_t key[2], int64_t num, int64_t n, int64_t ld, int32_t dtype,
                       void *out, void *stream) {
  if (!key || !out || n <= 0 || ld < n || ld % 8 != 0 || num < 0 || !aligned16(out))
    return MFG_ERR_BAD_ARG;
  cudaStream_t s = as_stream(stream);
  const double b = (double)num * ld * (dtype == MFG_F64 ? 8.0 : 4.0);
  if (dtype == MFG_F32)
    MFG_LAUNCH(MFG_PROF_OTHER, b, 0.0, launch_sampler<float>(1, key[0], key[1], num, n, ld, (float *)out, s));
  else if (dtype == MFG_F64)
    MFG_LAUNCH(MFG_PROF_OTHER, b, 0.0, launch_sampler<double>(1, key[0], key[1], num, n, ld, (double *)out, s));
  else
    return MFG_ERR_BAD_ARG;
  return MFG_OK;
}

int mfg_operator_apply(const mfg_operator *op, const void *V, void *W, int64_t p, int64_t ld,
                       void *workspace, size_t workspace_bytes, void *stream) {
  MFG_TRY(check_op(op));
  MFG_TRY(check_panel(op, p, ld));
  if (!V || !W || !aligned16(V) || !aligned16(W)) return MFG_ERR_BAD_ARG;
  const WsLayout L = layout(op, 0, p, ld);
  if (!workspace || workspace_bytes < L.total) return MFG_ERR_WORKSPACE;
  char *ws = ws_base(workspace);
  cudaStream_t s = as_stream(stream);
  int *status = reinterpret_cast<int *>(ws + L.status);
  if (op->precision == MFG_PREC_FP64)
    return apply_op<double>(op, (const double *)V, ld, (double *)W, ld, p, nullptr, nullptr, ld,
                            reinterpret_cast<double *>(ws + L.panel), status, s);
  __nv_bfloat16 *hi = nullptr, *lo = nullptr;
  if (uses_bf16(op)) {
    hi = reinterpret_cast<__nv_bfloat16 *>(ws + L.hi);
    lo = op->precision == MFG_PREC_BF16X3 ? reinterpret_cast<__nv_bfloat16 *>(ws + L.lo) : nullptr;
    MFG_TRY(launch_split_bf16((const float *)V, p, op->n, ld, hi, lo, ld, s));
  }
  return apply_op<float>(op, (const float *)V, ld, (float *)W, ld, p, hi, lo, ld,
                         reinterpret_cast<float *>(ws + L.panel), status, s);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Operator application without any allocation.
//
// The panel's bf16 copies go to a file-scope device array instead of a
// caller workspace.  In host code `g_noalloc_scratch` names a host-side shadow,
// not device memory, so its device address is looked up per device with
// cudaGetSymbolAddress (with that device current) on the first call there
// and cached.  Layout: [0, 256) status word, then hi, then lo.
// ---------------------------------------------------------------------------

static __device__ __align__(256) unsigned char g_noalloc_scratch[MFG_NOALLOC_SCRATCH_BYTES];

namespace mfg {
constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
static void *g_noalloc_ptr[kMaxDevices] = {nullptr};

static int noalloc_scratch(void **out) {
  int dev = 0;
  MFG_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return MFG_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || ptr == nullptr)
      return MFG_ERR_CUDA;
    g_noalloc_ptr[dev] = ptr;
  }
  *out = g_noalloc_ptr[dev];
  return MFG_OK;
}
}  // namespace mfg

extern "C" {

int mfg_operator_apply_noalloc(const mfg_operator *op, const void *V, void *W, int64_t p,
                               int64_t ld, void *stream) {
  MFG_TRY(check_op(op));
  MFG_TRY(check_panel(op, p, ld));
  if (!V || !W || !aligned16(V) || !aligned16(W)) return MFG_ERR_BAD_ARG;
  // scratch need: status word + bf16 hi (+ lo) copies of the panel
  const size_t copies = uses_bf16(op) ? (op->precision == MFG_PREC_BF16X3 ? 2 : 1) : 0;
  const size_t panel_bytes = align_up((size_t)p * (size_t)ld * 2, 256);
  if (256 + copies * panel_bytes > MFG_NOALLOC_SCRATCH_BYTES) return MFG_ERR_SCRATCH_LIMIT;
  void *base = nullptr;
  MFG_TRY(noalloc_scratch(&base));
  char *sc = reinterpret_cast<char *>(base);
  cudaStream_t s = as_stream(stream);
  int *status = reinterpret_cast<int *>(sc);
  MFG_CUDA_TRY(cudaMemsetAsync(status, 0, sizeof(int), s));
  if (op->precision == MFG_PREC_FP64)
    return apply_op<double>(op, (const double *)V, ld, (double *)W, ld, p, nullptr, nullptr, ld,
                            nullptr, status, s);
  __nv_bfloat16 *hi = nullptr, *lo = nullptr;
  if (copies > 0) {
    hi = reinterpret_cast<__nv_bfloat16 *>(sc + 256);
    lo = copies == 2 ? reinterpret_cast<__nv_bfloat16 *>(sc + 256 + panel_bytes) : nullptr;
    MFG_TRY(launch_split_bf16((const float *)V, p, op->n, ld, hi, lo, ld, s));
  }
  return apply_op<float>(op, (const float *)V, ld, (float *)W, ld, p, hi, lo, ld, nullptr, status, s);
}

int mfg_operator_apply_noalloc_status(void *stream) {
  void *base = nullptr;
  MFG_TRY(noalloc_scratch(&base));
  cudaStream_t s = as_stream(stream);
  int word = 0;
  MFG_CUDA_TRY(cudaMemcpyAsync(&word, base, sizeof(int), cudaMemcpyDeviceToHost, s));
  MFG_CUDA_TRY(cudaStreamSynchronize(s));
  return word;
}

int mfg_wait_selftest(uint64_t limit_ns, void *status, void *times, void *stream) {
  if (!status || !times) return MFG_ERR_BAD_ARG;
  if (limit_ns == 0 || limit_ns > kMbarWaitNs) return MFG_ERR_BAD_ARG;
  return launch_wait_selftest(limit_ns, static_cast<int *>(status),
                              static_cast<unsigned long long *>(times), as_stream(stream));
}

int mfg_hessenberg(const mfg_operator *op, int64_t k, int64_t p, const void *V, int64_t ld,
                   int32_t reortho, void *Q, double *H, void *residual, double *init_len_inv,
                   void *workspace, size_t workspace_bytes, void *stream) {
  MFG_TRY(check_op(op));
  MFG_TRY(check_panel(op, p, ld));
  if (k < 0 || k > op->n) return MFG_ERR_RANGE;
  if (!V || !aligned16(V) || (k > 0 && (!Q || !H || !aligned16(Q)))) return MFG_ERR_BAD_ARG;
  if (residual && !aligned16(residual)) return MFG_ERR_BAD_ARG;
  if (reortho < 0 || reortho > 3) return MFG_ERR_BAD_ARG;
  if (reortho == 3 && !two_sweep_applies(op, k)) reortho = 1;
  const WsLayout L = layout(op, k, p, ld, reortho == 3);
  if (!workspace || workspace_bytes < L.total) return MFG_ERR_WORKSPACE;
  char *ws = ws_base(workspace);
  cudaStream_t s = as_stream(stream);
  if (op->precision == MFG_PREC_FP64)
    return run_hessenberg<double>(op, k, p, (const double *)V, ld, reortho, (double *)Q, H,
                                  (double *)residual, init_len_inv, L, ws, s);
  return run_hessenberg<float>(op, k, p, (const float *)V, ld, reortho, (float *)Q, H,
                               (float *)residual, init_len_inv, L, ws, s);
}

size_t mfg_adjoint_workspace_bytes(const mfg_operator *op, int64_t k, int64_t p, int64_t ld) {
  if (check_op(op) != MFG_OK || k <= 0 || p <= 0 || ld < op->n) return 0;
  return adj_layout(op, k, p, ld).total;
}

int mfg_hessenberg_adjoint_ex(const mfg_operator *op, int64_t k, int64_t p, int64_t ld, const void *Q,
                              const double *H, const void *residual, const double *init_len_inv,
                              const void *dQ, const double *dH, const void *dr, const double *dc,
                              void *Lambda, void *dv, void *workspace, size_t workspace_bytes,
                              void *stream) {
  MFG_TRY(check_op(op));
  MFG_TRY(check_panel(op, p, ld));
  if (k == 0) return MFG_ERR_RANGE;  // decomp.py:483-486: not defined for num_matvecs = 0
  if (k < 0 || k > op->n) return MFG_ERR_RANGE;
  if (!Q || !H || !residual || !init_len_inv || !dH || !Lambda || !dv) return MFG_ERR_BAD_ARG;
  if (!aligned16(Q) || !aligned16(residual) || !aligned16(Lambda) || !aligned16(dv) ||
      (dr && !aligned16(dr)) || (dQ && !aligned16(dQ)))
    return MFG_ERR_BAD_ARG;
  const AdjLayout L = adj_layout(op, k, p, ld);
  if (!workspace || workspace_bytes < L.total) return MFG_ERR_WORKSPACE;
  char *ws = ws_base(workspace);
  cudaStream_t s = as_stream(stream);
  if (op->precision == MFG_PREC_FP64)
    return run_adjoint<double>(op, k, p, ld, (const double *)Q, H, (const double *)residual,
                               init_len_inv, (const double *)dQ, dH, (const double *)dr, dc,
                               (double *)Lambda, (double *)dv, L, ws, s);
  return run_adjoint<float>(op, k, p, ld, (const float *)Q, H, (const float *)residual, init_len_inv,
                            (const float *)dQ, dH, (const float *)dr, dc, (float *)Lambda, (float *)dv,
                            L, ws, s);
}

int mfg_hessenberg_adjoint(const mfg_operator *op, int64_t k, int64_t p, int64_t ld, const void *Q,
                           const double *H, const void *residual, const double *init_len_inv,
                           const double *dH, const void *dr, const double *dc, void *Lambda,
                           void *dv, void *workspace, size_t workspace_bytes, void *stream) {
  return mfg_hessenberg_adjoint_ex(op, k, p, ld, Q, H, residual, init_len_inv, nullptr, dH, dr, dc,
                                   Lambda, dv, workspace, workspace_bytes, stream);
}

int mfg_gemm_tuning_add(int64_t n_lo, int64_t n_hi, int64_t p_lo, int64_t p_hi, int32_t bn,
                        int32_t split_k) {
  return gemm_rule_add(n_lo, n_hi, p_lo, p_hi, bn, split_k);
}

int mfg_gemm_tuning_clear(void) { return gemm_rules_clear(); }

int mfg_basis_combine(int32_t dtype, int64_t k, int64_t p, int64_t n, int64_t ld, const void *Q,
                      const double *coef, void *out, void *stream) {
  if (k < 0 || p < 0 || n <= 0 || ld < n || ld % 8 != 0) return MFG_ERR_BAD_ARG;
  if (dtype != MFG_F32 && dtype != MFG_F64) return MFG_ERR_BAD_ARG;
  if (p == 0) return MFG_OK;
  if ((k > 0 && (!Q || !coef)) || !out || !aligned16(out) || (Q && !aligned16(Q))) return MFG_ERR_BAD_ARG;
  cudaStream_t s = as_stream(stream);
  const double es = dtype == MFG_F64 ? 8.0 : 4.0;
  if (dtype == MFG_F64)
    MFG_LAUNCH(MFG_PROF_SUB, es * (k + 1.0) * n * p, 2.0 * k * n * p,
               launch_basis_combine<double>((const double *)Q, k, ld, n, p, coef, (double *)out, s));
  else
    MFG_LAUNCH(MFG_PROF_SUB, es * (k + 1.0) * n * p, 2.0 * k * n * p,
               launch_basis_combine<float>((const float *)Q, k, ld, n, p, coef, (float *)out, s));
  return MFG_OK;
}

int mfg_tridiag_eigh(int64_t k, int64_t p, const double *H, double *eigvals, double *eigvecs,
                     double *scratch, void *stream) {
  if (k <= 0 || p <= 0 || !H || !eigvals || !eigvecs || !scratch) return MFG_ERR_BAD_ARG;
  cudaStream_t s = as_stream(stream);
  MFG_LAUNCH(MFG_PROF_QUAD, 8.0 * p * k * k * 3.0, 6.0 * p * k * k * k,
             launch_tridiag_eigh_full(k, p, H, eigvals, eigvecs, scratch, nullptr, s));
  return MFG_OK;
}

int mfg_tridiag_quadrature(int64_t k, int64_t p, const double *H, int32_t fun, double param,
                           const double *scale, double *values, double *eigvals, double *first_sq,
                           void *stream) {
  if (k <= 0 || p <= 0 || !H || fun < MFG_FUN_LOG || fun > MFG_FUN_NONE) return MFG_ERR_BAD_ARG;
  cudaStream_t s = as_stream(stream);
  MFG_LAUNCH(MFG_PROF_QUAD, 8.0 * p * k * k + 16.0 * p * k, 0.0,
             launch_tridiag_quadrature(k, p, H, fun, param, scale, values, eigvals, first_sq,
                                       nullptr, s));
  return MFG_OK;
}

static int slq_impl(const mfg_operator *op, int64_t k, int64_t p, const void *probes, int64_t ld,
                    int32_t fun, double param, double *values, double *mean_sem, void *Q,
                    double *H, bool two, void *workspace, size_t workspace_bytes, void *stream) {
  MFG_TRY(check_op(op));
  MFG_TRY(check_panel(op, p, ld));
  if (k < 0 || k > op->n) return MFG_ERR_RANGE;
  if (k == 0) return MFG_ERR_BAD_ARG;  // e1 of a 0 x 0 matrix does not exist
  if (!probes || !aligned16(probes) || !values) return MFG_ERR_BAD_ARG;
  if (fun < MFG_FUN_LOG || fun > MFG_FUN_POW) return MFG_ERR_BAD_ARG;
  two = two && two_sweep_applies(op, k);
  const WsLayout L = layout(op, k, p, ld, two);
  if (!workspace || workspace_bytes < L.total) return MFG_ERR_WORKSPACE;
  char *ws = ws_base(workspace);
  cudaStream_t s = as_stream(stream);
  void *Qb = Q ? Q : (void *)(ws + L.q);
  double *Hb = H ? H : reinterpret_cast<double *>(ws + L.h);
  double *len0 = reinterpret_cast<double *>(ws + L.len0);
  double *scale = reinterpret_cast<double *>(ws + L.values);
  int *status = reinterpret_cast<int *>(ws + L.status);
  if (Q && !aligned16(Q)) return MFG_ERR_BAD_ARG;
  if (op->precision == MFG_PREC_FP64)
    MFG_TRY(run_hessenberg<double>(op, k, p, (const double *)probes, ld, 1, (double *)Qb, Hb,
                                   nullptr, nullptr, L, ws, s));
  else
    MFG_TRY(run_hessenberg<float>(op, k, p, (const float *)probes, ld, two ? 3 : 1, (float *)Qb, Hb,
                                  nullptr, nullptr, L, ws, s));
  // funm.py:240-241: length^2 * e1^T f(T) e1 with length = ||v||
  MFG_LAUNCH(MFG_PROF_OTHER, 16.0 * p, (double)p, launch_square(len0, scale, p, s));
  MFG_LAUNCH(MFG_PROF_QUAD, 8.0 * p * k * k + 16.0 * p * k, 0.0,
             launch_tridiag_quadrature(k, p, Hb, fun, param, scale, values,
                                       reinterpret_cast<double *>(ws + L.eig),
                                       reinterpret_cast<double *>(ws + L.fsq), status, s));
  if (mean_sem) MFG_LAUNCH(MFG_PROF_QUAD, 8.0 * p, 3.0 * p, launch_mean_sem(values, p, mean_sem, s));
  return MFG_OK;
}

int mfg_slq(const mfg_operator *op, int64_t k, int64_t p, const void *probes, int64_t ld,
            int32_t fun, double param, double *values, double *mean_sem, void *Q, double *H,
            void *workspace, size_t workspace_bytes, void *stream) {
  return slq_impl(op, k, p, probes, ld, fun, param, values, mean_sem, Q, H, false, workspace,
                  workspace_bytes, stream);
}

size_t mfg_slq_ex_workspace_bytes(const mfg_operator *op, int64_t k, int64_t p, int64_t ld,
                                  int32_t flags) {
  if (check_op(op) != MFG_OK || k < 0 || p <= 0 || ld < op->n) return 0;
  return layout(op, k, p, ld, (flags & MFG_SLQ_TWO_SWEEP) && two_sweep_applies(op, k)).total;
}

int mfg_slq_ex(const mfg_operator *op, int64_t k, int64_t p, const void *probes, int64_t ld,
               int32_t fun, double param, double *values, double *mean_sem, void *Q, double *H,
               int32_t flags, void *workspace, size_t workspace_bytes, void *stream) {
  if (flags & ~MFG_SLQ_TWO_SWEEP) return MFG_ERR_BAD_ARG;
  return slq_impl(op, k, p, probes, ld, fun, param, values, mean_sem, Q, H,
                  (flags & MFG_SLQ_TWO_SWEEP) != 0, workspace, workspace_bytes, stream);
}

int mfg_workspace_status(const void *workspace, void *stream) {
  if (!workspace) return MFG_ERR_BAD_ARG;
  int st = MFG_OK;
  cudaStream_t s = as_stream(stream);
  MFG_CUDA_TRY(cudaMemcpyAsync(&st, ws_base(const_cast<void *>(workspace)), sizeof(int),
                               cudaMemcpyDeviceToHost, s));
  MFG_CUDA_TRY(cudaStreamSynchronize(s));
  return st;
}

static int check_bidiag_ops(const mfg_operator *A, const mfg_operator *At, int64_t p, int64_t ld) {
  MFG_TRY(check_op(A));
  MFG_TRY(check_op(At));
  if (A->n != At->n || elem_size_for(A) != elem_size_for(At)) return MFG_ERR_BAD_ARG;
  return check_panel(A, p, ld);
}

size_t mfg_bidiag_workspace_bytes(const mfg_operator *A, const mfg_operator *At, int64_t k,
                                  int64_t p, int64_t ld) {
  if (check_bidiag_ops(A, At, p, ld) != MFG_OK || k < 0 || k > A->n) return 0;
  return bidiag_layout(A, At, k, p, ld).total;
}

int mfg_bidiag(const mfg_operator *A, const mfg_operator *At, int64_t k, int64_t p, const void *V0,
               int64_t ld, void *U, void *V, double *alphas, double *betas, void *residual,
               double *init_len_inv, void *workspace, size_t workspace_bytes, void *stream) {
  MFG_TRY(check_bidiag_ops(A, At, p, ld));
  if (k < 0 || k > A->n) return MFG_ERR_RANGE;
  if (!V0 || !aligned16(V0) || (k > 0 && (!U || !V || !alphas || !betas))) return MFG_ERR_BAD_ARG;
  if ((U && !aligned16(U)) || (V && !aligned16(V)) || (residual && !aligned16(residual)))
    return MFG_ERR_BAD_ARG;
  const BidiagLayout L = bidiag_layout(A, At, k, p, ld);
  if (!workspace || workspace_bytes < L.total) return MFG_ERR_WORKSPACE;
  char *ws = ws_base(workspace);
  cudaStream_t s = as_stream(stream);
  if (A->precision == MFG_PREC_FP64)
    return run_bidiag<double>(A, At, k, p, (const double *)V0, ld, (double *)U, (double *)V, alphas,
                              betas, (double *)residual, init_len_inv, L, ws, s);
  return run_bidiag<float>(A, At, k, p, (const float *)V0, ld, (float *)U, (float *)V, alphas, betas,
                           (float *)residual, init_len_inv, L, ws, s);
}

int mfg_slq_product(const mfg_operator *A, const mfg_operator *At, int64_t k, int64_t p,
                    const void *probes, int64_t ld, int32_t fun, double param, double *values,
                    double *mean_sem, void *workspace, size_t workspace_bytes, void *stream) {
  MFG_TRY(check_bidiag_ops(A, At, p, ld));
  if (k < 1 || k > A->n) return MFG_ERR_RANGE;
  if (!probes || !aligned16(probes) || !values) return MFG_ERR_BAD_ARG;
  if (fun < MFG_FUN_LOG || fun > MFG_FUN_POW) return MFG_ERR_BAD_ARG;
  const BidiagLayout L = bidiag_layout(A, At, k, p, ld);
  if (!workspace || workspace_bytes < L.total) return MFG_ERR_WORKSPACE;
  char *ws = ws_base(workspace);
  cudaStream_t s = as_stream(stream);
  double *alphas = reinterpret_cast<double *>(ws + L.alphas);
  double *betas = reinterpret_cast<double *>(ws + L.betas);
  double *gram = reinterpret_cast<double *>(ws + L.gram);
  double *len0 = reinterpret_cast<double *>(ws + L.base.len0);
  double *scale = reinterpret_cast<double *>(ws + L.values);
  int *status = reinterpret_cast<int *>(ws + L.base.status);
  if (A->precision == MFG_PREC_FP64)
    MFG_TRY(run_bidiag<double>(A, At, k, p, (const double *)probes, ld, (double *)(ws + L.u),
                               (double *)(ws + L.v), alphas, betas, nullptr, nullptr, L, ws, s));
  else
    MFG_TRY(run_bidiag<float>(A, At, k, p, (const float *)probes, ld, (float *)(ws + L.u),
                              (float *)(ws + L.v), alphas, betas, nullptr, nullptr, L, ws, s));
  // funm.py:286-303: length^2 * e1^T f(B^T B) e1 through the eigenpairs of B^T B
  MFG_CUDA_TRY(cudaMemsetAsync(gram, 0, (size_t)p * k * k * 8, s));
  bidiag_gram_kernel<<<(unsigned)ceil_div(p * k, 128), 128, 0, s>>>(alphas, betas, k, p, gram);
  MFG_TRY(MFG_LAUNCH_STATUS());
  MFG_LAUNCH(MFG_PROF_OTHER, 16.0 * p, (double)p, launch_square(len0, scale, p, s));
  MFG_LAUNCH(MFG_PROF_QUAD, 8.0 * p * k * k + 16.0 * p * k, 0.0,
             launch_tridiag_quadrature(k, p, gram, fun, param, scale, values,
                                       reinterpret_cast<double *>(ws + L.base.eig),
                                       reinterpret_cast<double *>(ws + L.base.fsq), status, s));
  if (mean_sem) MFG_LAUNCH(MFG_PROF_QUAD, 8.0 * p, 3.0 * p, launch_mean_sem(values, p, mean_sem, s));
  return MFG_OK;
}

size_t mfg_cg_workspace_bytes(const mfg_operator *op, int64_t p, int64_t ld) {
  if (check_op(op) != MFG_OK || p <= 0 || ld < op->n) return 0;
  return cg_layout(op, p, ld).total;
}

int mfg_cg(const mfg_operator *op, int64_t p, const void *B, void *X, int64_t ld, double tol,
           double atol, int64_t maxiter, int32_t *iters, void *workspace, size_t workspace_bytes,
           void *stream) {
  MFG_TRY(check_op(op));
  MFG_TRY(check_panel(op, p, ld));
  if (!B || !X || !aligned16(B) || !aligned16(X) || tol < 0.0 || atol < 0.0) return MFG_ERR_BAD_ARG;
  if (op->kind == MFG_OP_CALLBACK && op->shift != 0.0) return MFG_ERR_UNSUPPORTED;
  const CgLayout L = cg_layout(op, p, ld);
  if (!workspace || workspace_bytes < L.total) return MFG_ERR_WORKSPACE;
  char *ws = ws_base(workspace);
  cudaStream_t s = as_stream(stream);
  if (maxiter <= 0) maxiter = 10 * op->n;  // jax.scipy.sparse.linalg.cg's default
  if (op->precision == MFG_PREC_FP64)
    return run_cg<double>(op, p, (const double *)B, (double *)X, ld, tol, atol, maxiter, iters, L, ws, s);
  return run_cg<float>(op, p, (const float *)B, (float *)X, ld, tol, atol, maxiter, iters, L, ws, s);
}

static int rbf_build(const float *x, int64_t n, int32_t dim, double s2, double ell,
                     int32_t precision, int dlogell, void *a, void *a_lo, int64_t lda, void *stream) {
  if (!x || !a || n <= 0 || dim <= 0 || lda < n || lda % 8 != 0 || ell <= 0.0) return MFG_ERR_BAD_ARG;
  if (precision == MFG_PREC_BF16X3 && !a_lo) return MFG_ERR_BAD_ARG;
  if (precision < MFG_PREC_FP32 || precision > MFG_PREC_FP64) return MFG_ERR_BAD_ARG;
  cudaStream_t s = as_stream(stream);
  const double es = precision == MFG_PREC_FP64 ? 8.0 : (precision == MFG_PREC_FP32 ? 4.0 : (precision == MFG_PREC_BF16X3 ? 4.0 : 2.0));
  MFG_LAUNCH(MFG_PROF_OTHER, (double)n * lda * es, 0.0,
             launch_rbf_build(x, n, dim, s2, ell, precision, dlogell, a, a_lo, lda, s));
  return MFG_OK;
}

int mfg_rbf_build(const float *x, int64_t n, int32_t dim, double s2, double ell,
                  int32_t precision, void *a, void *a_lo, int64_t lda, void *stream) {
  return rbf_build(x, n, dim, s2, ell, precision, 0, a, a_lo, lda, stream);
}

int mfg_rbf_build_dlogell(const float *x, int64_t n, int32_t dim, double s2, double ell,
                          int32_t precision, void *a, void *a_lo, int64_t lda, void *stream) {
  return rbf_build(x, n, dim, s2, ell, precision, 1, a, a_lo, lda, stream);
}

int mfg_split_bf16(const float *a, int64_t rows, int64_t cols, int64_t lda, void *hi, void *lo,
                   int64_t ld_out, void *stream) {
  if (!a || !hi || rows < 0 || cols < 0 || lda < cols || ld_out < cols) return MFG_ERR_BAD_ARG;
  return launch_split_bf16(a, rows, cols, lda, (__nv_bfloat16 *)hi, (__nv_bfloat16 *)lo, ld_out,
                           as_stream(stream));
}

}  // extern "C"
