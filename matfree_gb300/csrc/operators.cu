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
// Small tiles for operators whose large-tile grid would not fill the GPU
// (e.g. n = 1000, p = 100: 16 CTAs of 128 x 64 against 128 of 32 x 32).
template <typename T> struct SimtCfgSmall;
template <> struct SimtCfgSmall<float> {
  static constexpr int BM = 32, BP = 32, BK = 32, TM = 2, TP = 2;
};
template <> struct SimtCfgSmall<double> {
  static constexpr int BM = 32, BP = 32, BK = 16, TM = 2, TP = 2;
};

template <typename T, typename C>
__global__ void __launch_bounds__(256)
dense_simt_kernel(const T *__restrict__ A, int64_t lda, const T *__restrict__ V, int64_t ldv,
                  T *__restrict__ W, int64_t ldw, int64_t n, int64_t p, T shift) {
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
      if constexpr (TM % VW == 0 && TP % VW == 0) {
#pragma unroll
        for (int i = 0; i < TM; i += VW) vec_to_array<T>(*reinterpret_cast<const VT *>(&As[kk][tx * TM + i]), a + i);
#pragma unroll
        for (int j = 0; j < TP; j += VW) vec_to_array<T>(*reinterpret_cast<const VT *>(&Vs[kk][ty * TP + j]), v + j);
      } else {  // thread tiles narrower than a 16-byte vector
#pragma unroll
        for (int i = 0; i < TM; ++i) a[i] = As[kk][tx * TM + i];
#pragma unroll
        for (int j = 0; j < TP; ++j) v[j] = Vs[kk][ty * TP + j];
      }
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
  using CS = SimtCfgSmall<T>;
  if (n <= 0 || p <= 0) return MFG_OK;
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 152;
  }
  const int64_t gx = ceil_div(n, C::BM), gy = ceil_div(p, C::BP);
  if (gx * gy < sms) {
    const int64_t sy = ceil_div(p, CS::BP);
    if (sy > 65535) return MFG_ERR_UNSUPPORTED;
    dim3 grid((unsigned)ceil_div(n, CS::BM), (unsigned)sy);
    dense_simt_kernel<T, CS><<<grid, 256, 0, s>>>(A, lda, V, ldv, W, ldw, n, p, (T)shift);
    return MFG_LAUNCH_STATUS();
  }
  if (gy > 65535) return MFG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)gx, (unsigned)gy);
  dense_simt_kernel<T, C><<<grid, 256, 0, s>>>(A, lda, V, ldv, W, ldw, n, p, (T)shift);
  return MFG_LAUNCH_STATUS();
}
template int launch_dense_simt<float>(const float *, int64_t, const float *, int64_t, float *,
                                      int64_t, int64_t, int64_t, double, cudaStream_t);
template int launch_dense_simt<double>(const double *, int64_t, const double *, int64_t, double *,
                                       int64_t, int64_t, int64_t, double, cudaStream_t);

// ---------------------------------------------------------------------------
// CSR SpMM: W[b][r] = sum_e val[e] V[b][col[e]] + shift V[b][r]
//
// The panels are probe-major, so the product is p sparse matrix-vector
// products that share the CSR arrays.  The rows are cut into tiles of
// kWRows; CTAs take tiles round-robin, so neighbouring tiles run at the same
// time and the vector entries they share are served from L2.  (Equal tiles
// sized to a whole number of waves measured slower on the 2-D Laplacian: the
// smaller tiles re-read more of the neighbouring rows.)  Per tile:
//   1. each row thread (4 rows per thread, rows r0 + t + 256 i) loads the
//      first RMAX entries of its rows into registers once; the tile's column
//      range [lo, hi] (including its own rows, for the shift term) follows
//      from a block reduction;
//   2. when the range is at most kWMax entries (banded matrices: stencils of
//      bandwidth up to about (kWMax - kWRows) / 2), a copy warp streams probe
//      b's window V[b][lo..hi] into a ring of shared-memory buffers with one
//      1-D bulk copy (cp.async.bulk) per probe, and the row threads form every
//      product from registers and shared memory (one shared load and one FMA
//      per entry): each probe vector is read from HBM about once, in long
//      bursts, instead of as scattered 4-byte gathers;
//   3. otherwise (wide or random column patterns) the row threads gather from
//      global memory: lane = row for short rows, and a warp walks its rows
//      one at a time with a butterfly of warp shuffles when one of them is
//      longer than kWLong entries.
// Entries beyond RMAX of a row are read from global memory in the same order.
// Every sum runs in a fixed order, so results do not depend on timing.  All
// waits are bounded (MFG_ERR_TIMEOUT in *status); after a failure the CTA
// stops at the next tile boundary and drains its copies in flight.
// ---------------------------------------------------------------------------

constexpr int kWRows = 1024;                   // rows per tile
constexpr int kWThreads = 256;                 // row threads (8 warps) + one copy warp
constexpr int kWRowWarps = kWThreads / 32;
constexpr int kWRowsPerThread = kWRows / kWThreads;
constexpr int kWMax = 4096;                    // window entries per ring buffer (16 KB)
constexpr int kWStages = 6;
constexpr int kWLong = 32;                     // longer rows take the warp-cooperative path

struct WinShared {
  uint64_t full[kWStages];
  uint64_t empty[kWStages];
  int lo, hi, fail, pad;
  int32_t rp[kWRows + 4];
  float win[kWStages][kWMax];
};

__device__ __forceinline__ uint32_t sp_smem(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

template <int RMAX>
__global__ void __launch_bounds__(kWThreads + 32, RMAX <= 6 ? 2 : 1)
csr_spmm_window_kernel(const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                       const float *__restrict__ val, int64_t n, int tile_rows,
                       const float *__restrict__ V, int64_t ldv, float *__restrict__ W, int64_t ldw,
                       int64_t p, float shift, int *status) {
  extern __shared__ __align__(128) uint8_t sp_raw[];
  WinShared *sh = reinterpret_cast<WinShared *>(sp_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool copier = warp == kWRowWarps;
  volatile int *fail = &sh->fail;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kWStages; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sp_smem(&sh->full[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sp_smem(&sh->empty[s])),
                   "r"(kWRowWarps)
                   : "memory");
    }
    sh->fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const int64_t ntiles = (n + tile_rows - 1) / tile_rows;
  int64_t g = 0;          // window copies issued (copy warp) / consumed (row warps) by this CTA
  int64_t issued = 0;     // copy warp: for the drain after a failure
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    __syncthreads();  // the previous tile's shared data is no longer read
    if (*fail) break;  // uniform: read after the barrier
    const int64_t r0 = tile * tile_rows;
    const int rows = (int)(n - r0 < (int64_t)tile_rows ? n - r0 : (int64_t)tile_rows);
    for (int i = threadIdx.x; i <= rows; i += kWThreads + 32) sh->rp[i] = __ldg(rp + r0 + i);
    if (threadIdx.x == 0) {
      sh->lo = (int)r0;
      sh->hi = (int)(r0 + rows - 1);
    }
    __syncthreads();
    // this thread's rows: the first RMAX entries in registers
    int col[kWRowsPerThread][RMAX];
    float a[kWRowsPerThread][RMAX];
    int e0[kWRowsPerThread], len[kWRowsPerThread];
    if (!copier) {
      int cmin = 0x7fffffff, cmax = -1;
#pragma unroll
      for (int i = 0; i < kWRowsPerThread; ++i) {
        const int lr = threadIdx.x + i * kWThreads;
        e0[i] = lr < rows ? sh->rp[lr] : 0;
        len[i] = lr < rows ? sh->rp[lr + 1] - e0[i] : 0;
#pragma unroll
        for (int q = 0; q < RMAX; ++q) {
          col[i][q] = q < len[i] ? __ldg(ci + e0[i] + q) : (int)(r0 + (lr < rows ? lr : 0));
          a[i][q] = q < len[i] ? __ldg(val + e0[i] + q) : 0.f;
          if (q < len[i]) {
            cmin = min(cmin, col[i][q]);
            cmax = max(cmax, col[i][q]);
          }
        }
        for (int e = e0[i] + RMAX; e < e0[i] + len[i]; ++e) {
          const int c = __ldg(ci + e);
          cmin = min(cmin, c);
          cmax = max(cmax, c);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        cmin = min(cmin, __shfl_xor_sync(0xffffffffu, cmin, o));
        cmax = max(cmax, __shfl_xor_sync(0xffffffffu, cmax, o));
      }
      if (lane == 0) {
        atomicMin(&sh->lo, cmin);
        atomicMax(&sh->hi, cmax);
      }
    }
    __syncthreads();
    const int64_t lo = (int64_t)sh->lo & ~(int64_t)3;
    const int64_t wlen = ((int64_t)sh->hi + 1 - lo + 3) & ~(int64_t)3;  // <= ld - lo: ld % 8 == 0
    // (column indices outside [0, n) break the caller's contract; such a tile
    // never issues a bulk copy)
    const bool windowed = wlen <= kWMax && sh->lo >= 0 && sh->hi < n;

    if (windowed) {
      if (copier) {
        if (lane == 0) {
          int s = (int)(g % kWStages);
          uint32_t ph = (uint32_t)((g / kWStages) & 1);
          for (int64_t b = 0; b < p; ++b, ++g) {
            if (b > 0 && ++s == kWStages) {
              s = 0;
              ph ^= 1u;
            }
            if (g >= kWStages && !mbar_wait_bounded(sp_smem(&sh->empty[s]), ph ^ 1u, fail)) {
              *fail = 1;
              if (status) atomicExch(status, (int)MFG_ERR_TIMEOUT);
              break;
            }
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                             sp_smem(&sh->full[s])),
                         "r"((uint32_t)(wlen * 4))
                         : "memory");
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                ::"r"(sp_smem(&sh->win[s][0])), "l"(reinterpret_cast<uint64_t>(V + b * ldv + lo)),
                "r"((uint32_t)(wlen * 4)), "r"(sp_smem(&sh->full[s]))
                : "memory");
            issued = g + 1;
          }
        }
        g = __shfl_sync(0xffffffffu, g, 0);
        issued = __shfl_sync(0xffffffffu, issued, 0);
      } else {
        // byte offsets into the window: the columns, and each row's own entry
        const int lo32 = (int)lo;
        int self[kWRowsPerThread];
#pragma unroll
        for (int i = 0; i < kWRowsPerThread; ++i) {
          self[i] = 4 * (int)(r0 + threadIdx.x + i * kWThreads - lo32);
#pragma unroll
          for (int q = 0; q < RMAX; ++q) col[i][q] = 4 * (col[i][q] - lo32);
        }
        int s = (int)(g % kWStages);
        uint32_t ph = (uint32_t)((g / kWStages) & 1);
        for (int64_t b = 0; b < p; ++b, ++g) {
          const bool ok = !*fail && mbar_wait_bounded(sp_smem(&sh->full[s]), ph, fail);
          if (!ok) {
            if (lane == 0) {
              *fail = 1;
              if (status) atomicExch(status, (int)MFG_ERR_TIMEOUT);
            }
            break;
          }
          const char *w = reinterpret_cast<const char *>(sh->win[s]);
          float *Wb = W + b * ldw + r0 + threadIdx.x;
#pragma unroll
          for (int i = 0; i < kWRowsPerThread; ++i) {
            if ((int)threadIdx.x + i * kWThreads < rows) {
              float acc = shift * *reinterpret_cast<const float *>(w + self[i]);
#pragma unroll
              for (int q = 0; q < RMAX; ++q)
                acc = fmaf(a[i][q], *reinterpret_cast<const float *>(w + col[i][q]), acc);
              for (int e = e0[i] + RMAX; e < e0[i] + len[i]; ++e)
                acc = fmaf(__ldg(val + e), *reinterpret_cast<const float *>(w + 4 * (__ldg(ci + e) - lo32)), acc);
              Wb[i * kWThreads] = acc;
            }
          }
          __syncwarp();
          if (lane == 0)
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sp_smem(&sh->empty[s])) : "memory");
          if (++s == kWStages) {
            s = 0;
            ph ^= 1u;
          }
        }
      }
      continue;
    }

    // gather path
    if (copier) continue;
#pragma unroll 1
    for (int i = 0; i < kWRowsPerThread; ++i) {
      const int lr = threadIdx.x + i * kWThreads;
      const bool has_row = lr < rows;
      int lmax = len[i];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
      if (lmax <= kWLong) {
        const int64_t r = r0 + lr;
        for (int64_t b = 0; b < p; ++b) {
          if (has_row) {
            const float *Vb = V + b * ldv;
            float acc = shift * __ldg(Vb + r);
            for (int e = e0[i]; e < e0[i] + len[i]; ++e) acc = fmaf(__ldg(val + e), __ldg(Vb + __ldg(ci + e)), acc);
            W[b * ldw + r] = acc;
          }
        }
        continue;
      }
      // a long row among this warp's rows: the warp walks them one at a time
      for (int j = 0; j < 32; ++j) {
        const int lj = (lr - lane) + j;
        if (lj >= rows) break;
        const int f0 = sh->rp[lj], f1 = sh->rp[lj + 1];
        const int64_t r = r0 + lj;
        for (int64_t b = 0; b < p; ++b) {
          const float *Vb = V + b * ldv;
          float acc = 0.f;
          for (int e = f0 + lane; e < f1; e += 32) acc = fmaf(__ldg(val + e), __ldg(Vb + __ldg(ci + e)), acc);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          if (lane == 0) W[b * ldw + r] = fmaf(shift, __ldg(Vb + r), acc);
        }
      }
    }
  }
  // after a failure the copies in flight land before the shared memory goes away
  if (copier && lane == 0 && *fail) {
    for (int64_t t = (issued > kWStages ? issued - kWStages : 0); t < issued; ++t)
      mbar_wait_bounded(sp_smem(&sh->full[t % kWStages]), (uint32_t)((t / kWStages) & 1), nullptr,
                        kMbarWaitNs / 8);
  }
}

template <int RMAX>
static int launch_csr_spmm_t(const int32_t *row_ptr, const int32_t *col_idx, const float *val, int64_t n,
                             const float *V, int64_t ldv, float *W, int64_t ldw, int64_t p, double shift,
                             int *status, cudaStream_t s) {
  const size_t smem = sizeof(WinShared);
  static int per_sm = 0, sms = 0;
  if (per_sm == 0) {
    int dev = 0;
    MFG_CUDA_TRY(cudaGetDevice(&dev));
    MFG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MFG_CUDA_TRY(cudaFuncSetAttribute(csr_spmm_window_kernel<RMAX>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int q = 0;
    MFG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&q, csr_spmm_window_kernel<RMAX>,
                                                               kWThreads + 32, smem));
    if (q < 1) return MFG_ERR_UNSUPPORTED;
    per_sm = q;
  }
  const int64_t G = (int64_t)sms * per_sm;
  const int64_t tile_rows = kWRows;
  const int64_t ntiles = ceil_div(n, tile_rows);
  const int64_t grid = G < ntiles ? G : ntiles;
  csr_spmm_window_kernel<RMAX><<<(unsigned)grid, kWThreads + 32, smem, s>>>(
      row_ptr, col_idx, val, n, (int)tile_rows, V, ldv, W, ldw, p, (float)shift, status);
  return MFG_LAUNCH_STATUS();
}

int launch_csr_spmm(const int32_t *row_ptr, const int32_t *col_idx, const float *val, int64_t n,
                    int64_t nnz, const float *V, int64_t ldv, float *W, int64_t ldw, int64_t p,
                    double shift, int *status, cudaStream_t s) {
  if (n <= 0 || p <= 0) return MFG_OK;
  if (n > 0x7ffffff0 || ldv % 8 != 0 || reinterpret_cast<uintptr_t>(V) % 16 != 0) return MFG_ERR_UNSUPPORTED;
  // entries held in registers per row: 6 covers 2-D 5-point stencils, 12 the
  // 3-D 7-point ones and up to 12 entries; longer rows read the rest from
  // global memory
  if (nnz <= 6 * n)
    return launch_csr_spmm_t<6>(row_ptr, col_idx, val, n, V, ldv, W, ldw, p, shift, status, s);
  return launch_csr_spmm_t<12>(row_ptr, col_idx, val, n, V, ldv, W, ldw, p, shift, status, s);
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
  // this thread's 8 points in registers, read from shared memory once (a
  // read per row would be an 8-way bank conflict: threads are 8 floats
  // apart); dimensions past dim are zero on both sides and add nothing
  float xc[kRbfMaxDim][8];
#pragma unroll
  for (int d = 0; d < kRbfMaxDim; ++d)
#pragma unroll
    for (int e = 0; e < 8; ++e) xc[d][e] = d < dim ? xs[d][threadIdx.x * 8 + e] : 0.f;
  for (int rr = 0; rr < kRbfRows; ++rr) {
    const int64_t i = r0 + rr;
    if (i >= n) return;
    float xi[kRbfMaxDim];
#pragma unroll
    for (int d = 0; d < kRbfMaxDim; ++d) xi[d] = d < dim ? __ldg(x + i * dim + d) : 0.f;
    float v[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      float d2 = 0.f;
#pragma unroll
      for (int d = 0; d < kRbfMaxDim; ++d) {
        const float df = xi[d] - xc[d][e];
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
