// Operator kernels on CUDA cores: dense W = A V (float32 / float64), CSR
// SpMM, and builders of the dense RBF kernel matrix and its bf16 split.
#include "common.cuh"
#include "kernels.cuh"

namespace mfg {

// ---------------------------------------------------------------------------
// Dense W[b][m] = sum_k A[m][k] V[b][k] + shift V[b][m]  (CUDA cores)
//
// CTA tile: BM rows of A x BP probes, K in steps of BK staged through shared
// memory (A tile stored k-major so each thread reads its TM contiguous rows
// with 16-byte loads).  Global loads of the next K step are issued before
// the FMAs of the current one (register double buffering).
// ---------------------------------------------------------------------------

template <typename T> struct SimtCfg;
template <> struct SimtCfg<float> {
  static constexpr int BM = 128, BP = 64, BK = 16, TM = 8, TP = 4;
};
template <> struct SimtCfg<double> {
  static constexpr int BM = 128, BP = 64, BK = 8, TM = 8, TP = 4;
};

template <typename T>
__global__ void __launch_bounds__(256)
dense_simt_kernel(const T *__restrict__ A, int64_t lda, const T *__restrict__ V, int64_t ldv,
                  T *__restrict__ W, int64_t ldw, int64_t n, int64_t p, T shift) {
  using C = SimtCfg<T>;
  constexpr int BM = C::BM, BP = C::BP, BK = C::BK, TM = C::TM, TP = C::TP;
  constexpr int VW = Vec<T>::width;
  using VT = typename Vec<T>::type;
  constexpr int A_VECS = BM * BK / VW / 256;  // 16-byte loads per thread for the A tile
  constexpr int V_VECS = BP * BK / VW / 256;
  static_assert(A_VECS >= 1 && V_VECS >= 1, "tile too small for 256 threads");
  static_assert((BM / TM) * (BP / TP) == 256, "thread layout");
  __shared__ __align__(16) T As[BK][BM];
  __shared__ __align__(16) T Vs[BK][BP];

  const int t = threadIdx.x;
  const int tx = t % (BM / TM);  // row group
  const int ty = t / (BM / TM);  // probe group
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  const int64_t b0 = (int64_t)blockIdx.y * BP;

  T acc[TM][TP];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TP; ++j) acc[i][j] = (T)0;

  T ra[A_VECS][VW], rv[V_VECS][VW];
  auto gload = [&](int64_t k0) {
#pragma unroll
    for (int e = 0; e < A_VECS; ++e) {
      const int f = t + e * 256;
      const int row = f / (BK / VW), kq = (f % (BK / VW)) * VW;
      const int64_t m = m0 + row, kk = k0 + kq;
      if (m < n && kk + VW <= n) {
        vec_to_array<T>(__ldg(reinterpret_cast<const VT *>(A + m * lda + kk)), ra[e]);
      } else {
#pragma unroll
        for (int u = 0; u < VW; ++u) ra[e][u] = (m < n && kk + u < n) ? A[m * lda + kk + u] : (T)0;
      }
    }
#pragma unroll
    for (int e = 0; e < V_VECS; ++e) {
      const int f = t + e * 256;
      const int pb = f / (BK / VW), kq = (f % (BK / VW)) * VW;
      const int64_t b = b0 + pb, kk = k0 + kq;
      if (b < p && kk + VW <= n) {
        vec_to_array<T>(__ldg(reinterpret_cast<const VT *>(V + b * ldv + kk)), rv[e]);
      } else {
#pragma unroll
        for (int u = 0; u < VW; ++u) rv[e][u] = (b < p && kk + u < n) ? V[b * ldv + kk + u] : (T)0;
      }
    }
  };
  auto sstore = [&]() {
#pragma unroll
    for (int e = 0; e < A_VECS; ++e) {
      const int f = t + e * 256;
      const int row = f / (BK / VW), kq = (f % (BK / VW)) * VW;
#pragma unroll
      for (int u = 0; u < VW; ++u) As[kq + u][row] = ra[e][u];
    }
#pragma unroll
    for (int e = 0; e < V_VECS; ++e) {
      const int f = t + e * 256;
      const int pb = f / (BK / VW), kq = (f % (BK / VW)) * VW;
#pragma unroll
      for (int u = 0; u < VW; ++u) Vs[kq + u][pb] = rv[e][u];
    }
  };

  gload(0);
  for (int64_t k0 = 0; k0 < n; k0 += BK) {
    __syncthreads();
    sstore();
    __syncthreads();
    if (k0 + BK < n) gload(k0 + BK);
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[TM], v[TP];
#pragma unroll
      for (int i = 0; i < TM; i += VW) vec_to_array<T>(*reinterpret_cast<const VT *>(&As[kk][tx * TM + i]), a + i);
#pragma unroll
      for (int j = 0; j < TP; j += VW) vec_to_array<T>(*reinterpret_cast<const VT *>(&Vs[kk][ty * TP + j]), v + j);
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TP; ++j) acc[i][j] = fma(a[i], v[j], acc[i][j]);
    }
  }

#pragma unroll
  for (int j = 0; j < TP; ++j) {
    const int64_t b = b0 + ty * TP + j;
    if (b >= p) continue;
    const int64_t mb = m0 + tx * TM;
#pragma unroll
    for (int i = 0; i < TM; ++i) {
      const int64_t m = mb + i;
      if (m < n) W[b * ldw + m] = fma(shift, V[b * ldv + m], acc[i][j]);
    }
  }
}

template <typename T>
int launch_dense_simt(const T *A, int64_t lda, const T *V, int64_t ldv, T *W, int64_t ldw,
                      int64_t n, int64_t p, double shift, cudaStream_t s) {
  using C = SimtCfg<T>;
  if (n <= 0 || p <= 0) return MFG_OK;
  const int64_t gy = ceil_div(p, C::BP);
  if (gy > 65535) return MFG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)ceil_div(n, C::BM), (unsigned)gy);
  dense_simt_kernel<T><<<grid, 256, 0, s>>>(A, lda, V, ldv, W, ldw, n, p, (T)shift);
  return MFG_LAUNCH_STATUS();
}
template int launch_dense_simt<float>(const float *, int64_t, const float *, int64_t, float *,
                                      int64_t, int64_t, int64_t, double, cudaStream_t);
template int launch_dense_simt<double>(const double *, int64_t, const double *, int64_t, double *,
                                       int64_t, int64_t, int64_t, double, cudaStream_t);

// ---------------------------------------------------------------------------
// CSR SpMM: W[b][r] = sum_e val[e] V[b][col[e]] + shift V[b][r]
//
// One thread per (row, group of kPG probes); the probe group is the fastest
// grid index so the CTAs that share a row range (and its CSR segment) run
// together and the segment is served from L2 after its first read.  Lanes of
// a warp own consecutive rows, so for banded / stencil matrices the gathers
// of one probe are coalesced.
// ---------------------------------------------------------------------------

constexpr int kPG = 8;

__global__ void __launch_bounds__(256)
csr_spmm_kernel(const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                const float *__restrict__ val, int64_t n, const float *__restrict__ V,
                int64_t ldv, float *__restrict__ W, int64_t ldw, int64_t p, float shift) {
  const int64_t r = (int64_t)blockIdx.y * blockDim.x + threadIdx.x;
  const int64_t b0 = (int64_t)blockIdx.x * kPG;
  if (r >= n) return;
  float acc[kPG];
#pragma unroll
  for (int g = 0; g < kPG; ++g) acc[g] = (b0 + g < p) ? shift * __ldg(V + (b0 + g) * ldv + r) : 0.f;
  const int e0 = __ldg(rp + r), e1 = __ldg(rp + r + 1);
  for (int e = e0; e < e1; ++e) {
    const int64_t c = __ldg(ci + e);
    const float a = __ldg(val + e);
#pragma unroll
    for (int g = 0; g < kPG; ++g)
      if (b0 + g < p) acc[g] = fmaf(a, __ldg(V + (b0 + g) * ldv + c), acc[g]);
  }
#pragma unroll
  for (int g = 0; g < kPG; ++g)
    if (b0 + g < p) W[(b0 + g) * ldw + r] = acc[g];
}

int launch_csr_spmm(const int32_t *row_ptr, const int32_t *col_idx, const float *val, int64_t n,
                    const float *V, int64_t ldv, float *W, int64_t ldw, int64_t p, double shift,
                    cudaStream_t s) {
  if (n <= 0 || p <= 0) return MFG_OK;
  const int64_t gy = ceil_div(n, 256);
  const int64_t gx = ceil_div(p, kPG);
  if (gy > 65535 || gx > 65535) return MFG_ERR_UNSUPPORTED;
  csr_spmm_kernel<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, s>>>(row_ptr, col_idx, val, n, V,
                                                                   ldv, W, ldw, p, (float)shift);
  return MFG_LAUNCH_STATUS();
}

// ---------------------------------------------------------------------------
// RBF kernel matrix and bf16 split
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256)
rbf_kernel(const float *__restrict__ x, int64_t n, int dim, double s2, double inv2l2, int prec,
           int dlogell, void *__restrict__ a, void *__restrict__ a_lo, int64_t lda) {
  const int64_t i = blockIdx.y;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= lda) return;
  const int64_t o = i * lda + j;
  if (prec == MFG_PREC_FP64) {
    double v = 0.0;
    if (j < n) {
      double d2 = 0.0;
      for (int d = 0; d < dim; ++d) {
        const double df = (double)x[i * dim + d] - (double)x[j * dim + d];
        d2 += df * df;
      }
      v = s2 * exp(-d2 * inv2l2);
      if (dlogell) v *= 2.0 * d2 * inv2l2;  // d/dlog(ell) of exp(-d2/(2 ell^2))
    }
    reinterpret_cast<double *>(a)[o] = v;
    return;
  }
  float v = 0.f;
  if (j < n) {
    float d2 = 0.f;
    for (int d = 0; d < dim; ++d) {
      const float df = x[i * dim + d] - x[j * dim + d];
      d2 = fmaf(df, df, d2);
    }
    v = (float)s2 * expf(-d2 * (float)inv2l2);
    if (dlogell) v *= 2.f * d2 * (float)inv2l2;
  }
  if (prec == MFG_PREC_FP32) {
    reinterpret_cast<float *>(a)[o] = v;
  } else {
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    reinterpret_cast<__nv_bfloat16 *>(a)[o] = h;
    if (prec == MFG_PREC_BF16X3)
      reinterpret_cast<__nv_bfloat16 *>(a_lo)[o] = __float2bfloat16_rn(v - __bfloat162float(h));
  }
}

// fp32 / bf16 / bf16 hi+lo entries.  A CTA covers kRbfRows rows x 2048
// columns: the columns' points are staged in shared memory once (coalesced,
// coordinate-major) and reused for every row; each thread forms eight
// consecutive entries of a row and stores them with one 16-byte store per
// bf16 array (two for fp32).  Each entry is computed exactly as in rbf_kernel.
constexpr int kRbfRows = 16;
constexpr int kRbfCols = 256 * 8;
constexpr int kRbfMaxDim = 4;

__global__ void __launch_bounds__(256)
rbf8_kernel(const float *__restrict__ x, int64_t n, int dim, float s2, float inv2l2, int prec,
            int dlogell, void *__restrict__ a, void *__restrict__ a_lo, int64_t lda) {
  __shared__ __align__(16) float xs[kRbfMaxDim][kRbfCols];
  const int64_t c0 = (int64_t)blockIdx.x * kRbfCols;
  const int64_t r0 = (int64_t)blockIdx.y * kRbfRows;
  for (int t = threadIdx.x; t < kRbfCols * dim; t += 256) {
    const int c = t / dim, d = t - c * dim;  // x is point-major: coalesced reads
    const int64_t j = c0 + c;
    xs[d][c] = j < n ? x[j * dim + d] : 0.f;
  }
  __syncthreads();
  const int64_t j0 = c0 + (int64_t)threadIdx.x * 8;
  if (j0 >= lda) return;
  for (int rr = 0; rr < kRbfRows; ++rr) {
    const int64_t i = r0 + rr;
    if (i >= n) return;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      float d2 = 0.f;
      for (int d = 0; d < dim; ++d) {
        const float df = x[i * dim + d] - xs[d][threadIdx.x * 8 + e];
        d2 = fmaf(df, df, d2);
      }
      float w = s2 * expf(-d2 * inv2l2);
      if (dlogell) w *= 2.f * d2 * inv2l2;
      v[e] = (j0 + e < n) ? w : 0.f;
    }
    const int64_t o = i * lda + j0;  // 8-element aligned: lda % 8 == 0
    if (prec == MFG_PREC_FP32) {
      float4 *dst = reinterpret_cast<float4 *>(reinterpret_cast<float *>(a) + o);
      dst[0] = make_float4(v[0], v[1], v[2], v[3]);
      dst[1] = make_float4(v[4], v[5], v[6], v[7]);
      continue;
    }
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int e = 0; e < 8; e += 2) {
      const __nv_bfloat16 h0 = __float2bfloat16_rn(v[e]), h1 = __float2bfloat16_rn(v[e + 1]);
      hw[e / 2] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
      const __nv_bfloat16 l0 = __float2bfloat16_rn(v[e] - __bfloat162float(h0));
      const __nv_bfloat16 l1 = __float2bfloat16_rn(v[e + 1] - __bfloat162float(h1));
      lw[e / 2] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
    }
    *reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(a) + o) =
        make_uint4(hw[0], hw[1], hw[2], hw[3]);
    if (prec == MFG_PREC_BF16X3)
      *reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(a_lo) + o) =
          make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
}

int launch_rbf_build(const float *x, int64_t n, int dim, double s2, double ell, int precision,
                     int dlogell, void *a, void *a_lo, int64_t lda, cudaStream_t s) {
  if (n <= 0) return MFG_OK;
  if (n > 65535) return MFG_ERR_UNSUPPORTED;
  const double inv2l2 = 1.0 / (2.0 * ell * ell);
  if (precision != MFG_PREC_FP64 && dim <= kRbfMaxDim && lda % 8 == 0 && ((uintptr_t)a & 15) == 0 &&
      (a_lo == nullptr || ((uintptr_t)a_lo & 15) == 0)) {
    rbf8_kernel<<<dim3((unsigned)ceil_div(lda, kRbfCols), (unsigned)ceil_div(n, kRbfRows)), 256, 0, s>>>(
        x, n, dim, (float)s2, (float)inv2l2, precision, dlogell, a, a_lo, lda);
    return MFG_LAUNCH_STATUS();
  }
  rbf_kernel<<<dim3((unsigned)ceil_div(lda, 256), (unsigned)n), 256, 0, s>>>(
      x, n, dim, s2, inv2l2, precision, dlogell, a, a_lo, lda);
  return MFG_LAUNCH_STATUS();
}

__global__ void split_kernel(const float *__restrict__ a, int64_t rows, int64_t cols, int64_t lda,
                             __nv_bfloat16 *__restrict__ hi, __nv_bfloat16 *__restrict__ lo,
                             int64_t ldo) {
  const int64_t i = blockIdx.y;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows || j >= ldo) return;
  const float v = (j < cols) ? a[i * lda + j] : 0.f;
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  hi[i * ldo + j] = h;
  if (lo) lo[i * ldo + j] = __float2bfloat16_rn(v - __bfloat162float(h));
}

int launch_split_bf16(const float *a, int64_t rows, int64_t cols, int64_t lda, __nv_bfloat16 *hi,
                      __nv_bfloat16 *lo, int64_t ld_out, cudaStream_t s) {
  if (rows <= 0) return MFG_OK;
  if (rows > 65535) return MFG_ERR_UNSUPPORTED;
  split_kernel<<<dim3((unsigned)ceil_div(ld_out, 256), (unsigned)rows), 256, 0, s>>>(
      a, rows, cols, lda, hi, lo, ld_out);
  return MFG_LAUNCH_STATUS();
}

}  // namespace mfg
