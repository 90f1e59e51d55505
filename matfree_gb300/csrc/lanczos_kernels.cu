// Streaming kernels of the batched Arnoldi / CGS2 step and the probe sampler.
//
// Layout: probe-major panels (probe b's vector is row b, ld elements apart);
// the basis of p probes holds k rows per probe.  Each CTA of the sweep
// kernels owns one contiguous chunk of one probe's rows, so every load is a
// coalesced 16-byte vector load and every reduction is over a contiguous
// range.  Dot products multiply in the data type, sum each thread's few
// products in that type, and combine across threads, warps and CTAs in
// float64; the cross-CTA sum runs in a fixed order (last-arriving CTA of a
// probe reduces all chunk partials), so results are deterministic.
#include "common.cuh"
#include "kernels.cuh"

namespace mfg {

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC 2011) and the probe samplers
// ---------------------------------------------------------------------------

struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    const uint32_t lo0 = 0xD2511F53u * c.x;
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
  }
  return c;
}

// One thread per 4 consecutive elements of one probe: counter (m, b, stream, 0).
template <typename T, int kStream>
__global__ void sampler_kernel(uint32_t k0, uint32_t k1, int64_t num, int64_t n, int64_t ld,
                               T *__restrict__ out) {
  const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t b = blockIdx.y;
  const int64_t mlim = (ld + 3) / 4;
  if (m >= mlim || b >= num) return;
  const U4 w = philox4x32_10(U4{(uint32_t)m, (uint32_t)b, (uint32_t)kStream, 0u}, k0, k1);
  T v[4];
  if (kStream == 0) {
    v[0] = (T)(1 - 2 * (int)(w.x >> 31));
    v[1] = (T)(1 - 2 * (int)(w.y >> 31));
    v[2] = (T)(1 - 2 * (int)(w.z >> 31));
    v[3] = (T)(1 - 2 * (int)(w.w >> 31));
  } else {
    // Box-Muller: u1 in (0, 1], u2 in [0, 1)
    const float u1a = ((float)w.x + 1.0f) * 2.3283064365386963e-10f;
    const float u2a = (float)w.y * 2.3283064365386963e-10f;
    const float u1b = ((float)w.z + 1.0f) * 2.3283064365386963e-10f;
    const float u2b = (float)w.w * 2.3283064365386963e-10f;
    const float ra = sqrtf(-2.0f * logf(u1a));
    const float rb = sqrtf(-2.0f * logf(u1b));
    float sa, ca, sb, cb;
    sincospif(2.0f * u2a, &sa, &ca);
    sincospif(2.0f * u2b, &sb, &cb);
    v[0] = (T)(ra * ca); v[1] = (T)(ra * sa); v[2] = (T)(rb * cb); v[3] = (T)(rb * sb);
  }
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int64_t i = 4 * m + t;
    if (i < ld) out[b * ld + i] = (i < n) ? v[t] : (T)0;
  }
}

template <typename T>
int launch_sampler(int stream_id, uint32_t k0, uint32_t k1, int64_t num, int64_t n, int64_t ld,
                   T *out, cudaStream_t s) {
  if (num <= 0 || n <= 0) return MFG_OK;
  const int64_t mlim = (ld + 3) / 4;
  dim3 grid((unsigned)ceil_div(mlim, kThreads), (unsigned)num);
  if (num > 65535) return MFG_ERR_UNSUPPORTED;
  if (stream_id == 0)
    sampler_kernel<T, 0><<<grid, kThreads, 0, s>>>(k0, k1, num, n, ld, out);
  else
    sampler_kernel<T, 1><<<grid, kThreads, 0, s>>>(k0, k1, num, n, ld, out);
  return cudaGetLastError() == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}
template int launch_sampler<float>(int, uint32_t, uint32_t, int64_t, int64_t, int64_t, float *, cudaStream_t);
template int launch_sampler<double>(int, uint32_t, uint32_t, int64_t, int64_t, int64_t, double *, cudaStream_t);

// ---------------------------------------------------------------------------
// Chunked, masked vector access
// ---------------------------------------------------------------------------

// Vectors per thread in one chunk; a chunk is kThreads * kVPT * width rows.
constexpr int kVPT = 2;

template <typename T> __host__ __device__ constexpr int chunk_rows() {
  return kThreads * kVPT * Vec<T>::width;
}

// Load the thread's kVPT vectors of row-range chunk `c`; elements at or
// beyond n read as zero.  Padding up to ld is in bounds because ld % 8 == 0.
// kReadOnly selects the non-coherent read-only path (data not written by the
// running kernel); the in-place update reads its vector with plain loads.
template <typename T, bool kReadOnly = true>
__device__ __forceinline__ void load_chunk(const T *base, int64_t n, int64_t c,
                                           T (&x)[kVPT][Vec<T>::width]) {
  constexpr int W = Vec<T>::width;
  using V = typename Vec<T>::type;
#pragma unroll
  for (int e = 0; e < kVPT; ++e) {
    const int64_t r = c * chunk_rows<T>() + ((int64_t)e * kThreads + threadIdx.x) * W;
    if (r < n) {
      const V *ptr = reinterpret_cast<const V *>(base + r);
      const V v = kReadOnly ? __ldg(ptr) : *ptr;
      vec_to_array<T>(v, x[e]);
#pragma unroll
      for (int q = 0; q < W; ++q)
        if (r + q >= n) x[e][q] = (T)0;
    } else {
#pragma unroll
      for (int q = 0; q < W; ++q) x[e][q] = (T)0;
    }
  }
}

template <typename T>
__device__ __forceinline__ void store_chunk(T *__restrict__ base, int64_t n, int64_t c,
                                            const T (&x)[kVPT][Vec<T>::width]) {
  constexpr int W = Vec<T>::width;
#pragma unroll
  for (int e = 0; e < kVPT; ++e) {
    const int64_t r = c * chunk_rows<T>() + ((int64_t)e * kThreads + threadIdx.x) * W;
    if (r < n) *reinterpret_cast<typename Vec<T>::type *>(base + r) = array_to_vec<T>(x[e]);
  }
}

// Deterministic cross-CTA finish: the last CTA of probe b (by arrival order)
// sums partials[b][0..nchunks)[i] in chunk order.  Returns true in that CTA.
__device__ __forceinline__ bool arrive_last(unsigned *counters, int64_t b, int nchunks) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned ticket = atomicAdd(&counters[b], 1u);
    s_last = (ticket == (unsigned)(nchunks - 1));
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// ---------------------------------------------------------------------------
// Projection h = Q^T w  (first and second Gram-Schmidt pass)
// ---------------------------------------------------------------------------

constexpr int kColGroup = 8;  // columns reduced together (independent loads in flight)

template <typename T>
__global__ void __launch_bounds__(kThreads)
proj_kernel(const T *__restrict__ Q, int64_t q_bstride, int64_t q_istride, int ncols,
            const T *__restrict__ Wv, int64_t w_bstride, int64_t n, int nchunks,
            double *__restrict__ partials, unsigned *__restrict__ counters,
            double *__restrict__ out, int64_t out_bstride, int64_t out_istride) {
  constexpr int W = Vec<T>::width;
  __shared__ double red[kColGroup][kWarps];
  const int64_t c = blockIdx.x;
  const int64_t b = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  T w[kVPT][W];
  load_chunk<T>(Wv + b * w_bstride, n, c, w);

  for (int i0 = 0; i0 < ncols; i0 += kColGroup) {
    double s[kColGroup];
#pragma unroll
    for (int g = 0; g < kColGroup; ++g) {
      T acc = (T)0;
      if (i0 + g < ncols) {
        T q[kVPT][W];
        load_chunk<T>(Q + b * q_bstride + (int64_t)(i0 + g) * q_istride, n, c, q);
#pragma unroll
        for (int e = 0; e < kVPT; ++e)
#pragma unroll
          for (int u = 0; u < W; ++u) acc = fma(q[e][u], w[e][u], acc);
      }
      s[g] = (double)acc;
    }
#pragma unroll
    for (int g = 0; g < kColGroup; ++g) s[g] = warp_sum(s[g]);
    if (lane == 0) {
#pragma unroll
      for (int g = 0; g < kColGroup; ++g) red[g][warp] = s[g];
    }
    __syncthreads();
    if (threadIdx.x < kColGroup && i0 + (int)threadIdx.x < ncols) {
      double t = 0.0;
#pragma unroll
      for (int q = 0; q < kWarps; ++q) t += red[threadIdx.x][q];
      const int i = i0 + threadIdx.x;
      if (nchunks == 1)
        out[b * out_bstride + i * out_istride] = t;
      else
        partials[(b * nchunks + c) * ncols + i] = t;
    }
    __syncthreads();
  }
  if (nchunks == 1) return;
  if (arrive_last(counters, b, nchunks)) {
    for (int i = threadIdx.x; i < ncols; i += kThreads) {
      double t = 0.0;
      for (int cc = 0; cc < nchunks; ++cc) t += __ldcg(&partials[(b * nchunks + cc) * ncols + i]);
      out[b * out_bstride + i * out_istride] = t;
    }
    if (threadIdx.x == 0) counters[b] = 0u;
  }
}

// ---------------------------------------------------------------------------
// Update w -= Q c, optionally with ||w|| (float64) fused
// ---------------------------------------------------------------------------

template <typename T, bool kNorm, bool kStore>
__global__ void __launch_bounds__(kThreads)
sub_kernel(const T *__restrict__ Q, int64_t q_bstride, int64_t q_istride, int ncols,
           const double *__restrict__ coef, int64_t c_bstride, int64_t c_istride,
           const T *Win, T *Wout, int64_t w_bstride, int64_t n,
           int nchunks, double *__restrict__ partials, unsigned *__restrict__ counters,
           double *__restrict__ norm_out, double *__restrict__ norm_out2,
           int64_t norm2_bstride) {
  constexpr int W = Vec<T>::width;
  extern __shared__ double s_coef_raw[];
  T *s_coef = reinterpret_cast<T *>(s_coef_raw);
  __shared__ double red[kWarps];
  const int64_t c = blockIdx.x;
  const int64_t b = blockIdx.y;

  for (int i = threadIdx.x; i < ncols; i += kThreads) s_coef[i] = (T)coef[b * c_bstride + i * c_istride];
  __syncthreads();

  T w[kVPT][W];
  load_chunk<T, false>(Win + b * w_bstride, n, c, w);
  int i = 0;
  for (; i + 4 <= ncols; i += 4) {
    T q0[kVPT][W], q1[kVPT][W], q2[kVPT][W], q3[kVPT][W];
    const T *qb = Q + b * q_bstride + (int64_t)i * q_istride;
    load_chunk<T>(qb, n, c, q0);
    load_chunk<T>(qb + q_istride, n, c, q1);
    load_chunk<T>(qb + 2 * q_istride, n, c, q2);
    load_chunk<T>(qb + 3 * q_istride, n, c, q3);
    const T c0 = s_coef[i], c1 = s_coef[i + 1], c2 = s_coef[i + 2], c3 = s_coef[i + 3];
#pragma unroll
    for (int e = 0; e < kVPT; ++e)
#pragma unroll
      for (int u = 0; u < W; ++u) {
        T x = w[e][u];
        x = fma(-q0[e][u], c0, x);
        x = fma(-q1[e][u], c1, x);
        x = fma(-q2[e][u], c2, x);
        x = fma(-q3[e][u], c3, x);
        w[e][u] = x;
      }
  }
  for (; i < ncols; ++i) {
    T q0[kVPT][W];
    load_chunk<T>(Q + b * q_bstride + (int64_t)i * q_istride, n, c, q0);
    const T c0 = s_coef[i];
#pragma unroll
    for (int e = 0; e < kVPT; ++e)
#pragma unroll
      for (int u = 0; u < W; ++u) w[e][u] = fma(-q0[e][u], c0, w[e][u]);
  }
  if (kStore) store_chunk<T>(Wout + b * w_bstride, n, c, w);
  if (!kNorm) return;

  T acc = (T)0;
#pragma unroll
  for (int e = 0; e < kVPT; ++e)
#pragma unroll
    for (int u = 0; u < W; ++u) acc = fma(w[e][u], w[e][u], acc);
  double sd = warp_sum((double)acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sd;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < kWarps; ++q) t += red[q];
    if (nchunks == 1) {
      const double nv = sqrt(t);
      norm_out[b] = nv;
      if (norm_out2) norm_out2[b * norm2_bstride] = nv;
    } else {
      partials[b * nchunks + c] = t;
    }
  }
  if (nchunks == 1) return;
  if (arrive_last(counters, b, nchunks)) {
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int cc = 0; cc < nchunks; ++cc) t += __ldcg(&partials[b * nchunks + cc]);
      const double nv = sqrt(t);
      norm_out[b] = nv;
      if (norm_out2) norm_out2[b * norm2_bstride] = nv;
      counters[b] = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// Normalise: out = w / norm (the reference's ``v /= length``), with optional
// bf16 hi/lo copies for the tensor-core operator.
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(kThreads)
scale_kernel(const T *__restrict__ Win, int64_t w_bstride, int64_t n, const double *__restrict__ norm,
             T *__restrict__ out, int64_t out_bstride, __nv_bfloat16 *__restrict__ hi,
             __nv_bfloat16 *__restrict__ lo, int64_t bf_bstride) {
  constexpr int W = Vec<T>::width;
  const int64_t c = blockIdx.x;
  const int64_t b = blockIdx.y;
  const T nv = (T)norm[b];
  T w[kVPT][W];
  load_chunk<T>(Win + b * w_bstride, n, c, w);
#pragma unroll
  for (int e = 0; e < kVPT; ++e)
#pragma unroll
    for (int u = 0; u < W; ++u) w[e][u] = w[e][u] / nv;
  store_chunk<T>(out + b * out_bstride, n, c, w);
  if (hi == nullptr) return;
#pragma unroll
  for (int e = 0; e < kVPT; ++e) {
    const int64_t r = c * chunk_rows<T>() + ((int64_t)e * kThreads + threadIdx.x) * W;
    if (r >= n) continue;
    __nv_bfloat16 h[W], l[W];
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const float x = (float)w[e][u];
      h[u] = __float2bfloat16_rn(x);
      l[u] = __float2bfloat16_rn(x - __bfloat162float(h[u]));
    }
#pragma unroll
    for (int u = 0; u < W; ++u) {
      hi[b * bf_bstride + r + u] = h[u];
      if (lo) lo[b * bf_bstride + r + u] = l[u];
    }
  }
}

__global__ void inv_kernel(const double *__restrict__ x, double *__restrict__ y, int64_t p) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b < p) y[b] = 1.0 / x[b];
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------

template <typename T>
int64_t num_chunks(int64_t n) { return ceil_div(n, chunk_rows<T>()); }
template int64_t num_chunks<float>(int64_t);
template int64_t num_chunks<double>(int64_t);

template <typename T>
int launch_proj(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols, const T *Wv,
                int64_t w_bstride, int64_t n, int64_t p, double *partials, unsigned *counters,
                double *out, int64_t out_bstride, int64_t out_istride, cudaStream_t s) {
  if (ncols <= 0 || p <= 0) return MFG_OK;
  const int64_t nch = num_chunks<T>(n);
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)nch, (unsigned)p);
  proj_kernel<T><<<grid, kThreads, 0, s>>>(Q, q_bstride, q_istride, ncols, Wv, w_bstride, n,
                                           (int)nch, partials, counters, out, out_bstride,
                                           out_istride);
  return cudaGetLastError() == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}

template <typename T>
int launch_sub(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols, const double *coef,
               int64_t c_bstride, int64_t c_istride, const T *Win, T *Wout, int64_t w_bstride,
               int64_t n, int64_t p, bool with_norm, bool store, double *partials,
               unsigned *counters, double *norm_out, double *norm_out2, int64_t norm2_bstride,
               cudaStream_t s) {
  if (p <= 0) return MFG_OK;
  const int64_t nch = num_chunks<T>(n);
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)nch, (unsigned)p);
  const size_t smem = (size_t)(ncols > 0 ? ncols : 1) * sizeof(T);
  if (smem > 48 * 1024) return MFG_ERR_UNSUPPORTED;
  if (with_norm && store)
    sub_kernel<T, true, true><<<grid, kThreads, smem, s>>>(
        Q, q_bstride, q_istride, ncols, coef, c_bstride, c_istride, Win, Wout, w_bstride, n,
        (int)nch, partials, counters, norm_out, norm_out2, norm2_bstride);
  else if (with_norm)
    sub_kernel<T, true, false><<<grid, kThreads, smem, s>>>(
        Q, q_bstride, q_istride, ncols, coef, c_bstride, c_istride, Win, Wout, w_bstride, n,
        (int)nch, partials, counters, norm_out, norm_out2, norm2_bstride);
  else
    sub_kernel<T, false, true><<<grid, kThreads, smem, s>>>(
        Q, q_bstride, q_istride, ncols, coef, c_bstride, c_istride, Win, Wout, w_bstride, n,
        (int)nch, partials, counters, norm_out, norm_out2, norm2_bstride);
  return cudaGetLastError() == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}

template <typename T>
int launch_scale(const T *Win, int64_t w_bstride, int64_t n, int64_t p, const double *norm, T *out,
                 int64_t out_bstride, __nv_bfloat16 *hi, __nv_bfloat16 *lo, int64_t bf_bstride,
                 cudaStream_t s) {
  if (p <= 0) return MFG_OK;
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)num_chunks<T>(n), (unsigned)p);
  scale_kernel<T><<<grid, kThreads, 0, s>>>(Win, w_bstride, n, norm, out, out_bstride, hi, lo,
                                            bf_bstride);
  return cudaGetLastError() == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}

int launch_inv(const double *x, double *y, int64_t p, cudaStream_t s) {
  if (p <= 0) return MFG_OK;
  inv_kernel<<<(unsigned)ceil_div(p, 128), 128, 0, s>>>(x, y, p);
  return cudaGetLastError() == cudaSuccess ? MFG_OK : MFG_ERR_CUDA;
}

#define MFG_INST(T)                                                                          \
  template int launch_proj<T>(const T *, int64_t, int64_t, int, const T *, int64_t, int64_t,   \
                              int64_t, double *, unsigned *, double *, int64_t, int64_t,       \
                              cudaStream_t);                                                   \
  template int launch_sub<T>(const T *, int64_t, int64_t, int, const double *, int64_t,        \
                             int64_t, const T *, T *, int64_t, int64_t, int64_t, bool, bool,   \
                             double *, unsigned *, double *, double *, int64_t, cudaStream_t); \
  template int launch_scale<T>(const T *, int64_t, int64_t, int64_t, const double *, T *,      \
                               int64_t, __nv_bfloat16 *, __nv_bfloat16 *, int64_t, cudaStream_t);
MFG_INST(float)
MFG_INST(double)
#undef MFG_INST

}  // namespace mfg
