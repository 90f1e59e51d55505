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
#include <cuda.h>

#include <cstdio>

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
  return MFG_LAUNCH_STATUS();
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
// ncols * kWarps doubles of dynamic shared memory must stay under the default
// 48 KB minus the kernels' static shared memory
constexpr int kMaxProjCols = 640;  // 40 KB dynamic + ~2.2 KB static

// Warp tree in the data type: one warp partial sums 32 lanes' products.
template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum the nred per-warp partials red[i][0..nred) of this CTA (float64) and
// finish the cross-CTA reduction of column i for probe b.
__device__ __forceinline__ void finish_columns(const double *red, int ncols, int64_t b, int64_t c,
                                               int nchunks, double *partials, unsigned *counters,
                                               double *out, int64_t out_bstride,
                                               int64_t out_istride, int nred = kWarps) {
  for (int i = threadIdx.x; i < ncols; i += kThreads) {
    double t = 0.0;
    for (int q = 0; q < nred; ++q) t += red[i * nred + q];
    if (nchunks == 1)
      out[b * out_bstride + i * out_istride] = t;
    else
      partials[(b * nchunks + c) * ncols + i] = t;
  }
  if (nchunks == 1) return;
  if (arrive_last(counters, b, nchunks)) {
    // G threads per column sum strided chunk partials, then a fixed-order
    // tree over those G sums: the last CTA's reduction is parallel and the
    // result does not depend on timing.
    __shared__ double s_red[kThreads];
    int G = 1;
    while (G < 32 && 2 * G * ncols <= kThreads && G < nchunks) G *= 2;
    const int cols_per_pass = kThreads / G;
    const int g = threadIdx.x % G;
    for (int i0 = 0; i0 < ncols; i0 += cols_per_pass) {
      const int i = i0 + (int)threadIdx.x / G;
      double t = 0.0;
      if (i < ncols) {
#pragma unroll 4
        for (int cc = g; cc < nchunks; cc += G) t += __ldcg(&partials[(b * nchunks + cc) * ncols + i]);
      }
      s_red[threadIdx.x] = t;
      __syncthreads();
      for (int st = G / 2; st > 0; st >>= 1) {
        if (g < st) s_red[threadIdx.x] += s_red[threadIdx.x + st];
        __syncthreads();
      }
      if (g == 0 && i < ncols) out[b * out_bstride + i * out_istride] = s_red[threadIdx.x];
      __syncthreads();
    }
    if (threadIdx.x == 0) counters[b] = 0u;
  }
}

// h = Q^T w for the first ncols basis vectors.  Each thread forms kVPT*width
// products per column in the data type, a warp sums its 32 lanes in the data
// type (256 products), and warps, chunks and the final value are combined in
// float64.  Warps run through the columns without block barriers; their
// partials meet in shared memory once at the end.
template <typename T>
__global__ void __launch_bounds__(kThreads)
proj_kernel(const T *__restrict__ Q, int64_t q_bstride, int64_t q_istride, int ncols,
            const T *__restrict__ Wv, int64_t w_bstride, int64_t n, int nchunks,
            double *__restrict__ partials, unsigned *__restrict__ counters,
            double *__restrict__ out, int64_t out_bstride, int64_t out_istride) {
  constexpr int W = Vec<T>::width;
  extern __shared__ double red[];  // [ncols][kWarps]
  const int64_t c = blockIdx.x;
  const int64_t b = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  T w[kVPT][W];
  load_chunk<T>(Wv + b * w_bstride, n, c, w);

  for (int i0 = 0; i0 < ncols; i0 += kColGroup) {
    T s[kColGroup];
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
      s[g] = acc;
    }
#pragma unroll
    for (int g = 0; g < kColGroup; ++g) s[g] = warp_sum_t<T>(s[g]);
    if (lane == 0) {
#pragma unroll
      for (int g = 0; g < kColGroup; ++g)
        if (i0 + g < ncols) red[(i0 + g) * kWarps + warp] = (double)s[g];
    }
  }
  __syncthreads();
  finish_columns(red, ncols, b, c, nchunks, partials, counters, out, out_bstride, out_istride);
}

// Shared-memory address and bulk-copy constants of the fused second pass
// (streamed kernel below).
__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

constexpr int kSPGroup = 8;  // basis vectors per 2-D tensor copy

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
    // strided per-thread sums, then a fixed-order tree (deterministic)
    __shared__ double s_red[kThreads];
    double t = 0.0;
#pragma unroll 4
    for (int cc = threadIdx.x; cc < nchunks; cc += kThreads) t += __ldcg(&partials[b * nchunks + cc]);
    s_red[threadIdx.x] = t;
    __syncthreads();
    for (int st = kThreads / 2; st > 0; st >>= 1) {
      if ((int)threadIdx.x < st) s_red[threadIdx.x] += s_red[threadIdx.x + st];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const double nv = sqrt(s_red[0]);
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
    if constexpr (W == 4) {
      // four bf16 per 8-byte store (r is a multiple of 4, the rows 16-byte aligned)
      uint2 hv, lv;
      hv.x = (uint32_t)__bfloat16_as_ushort(h[0]) | ((uint32_t)__bfloat16_as_ushort(h[1]) << 16);
      hv.y = (uint32_t)__bfloat16_as_ushort(h[2]) | ((uint32_t)__bfloat16_as_ushort(h[3]) << 16);
      lv.x = (uint32_t)__bfloat16_as_ushort(l[0]) | ((uint32_t)__bfloat16_as_ushort(l[1]) << 16);
      lv.y = (uint32_t)__bfloat16_as_ushort(l[2]) | ((uint32_t)__bfloat16_as_ushort(l[3]) << 16);
      *reinterpret_cast<uint2 *>(hi + b * bf_bstride + r) = hv;
      if (lo) *reinterpret_cast<uint2 *>(lo + b * bf_bstride + r) = lv;
    } else {
#pragma unroll
      for (int u = 0; u < W; ++u) {
        hi[b * bf_bstride + r + u] = h[u];
        if (lo) lo[b * bf_bstride + r + u] = l[u];
      }
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


// ---------------------------------------------------------------------------
// Fused second pass of CGS2: w' = w - Q h1 and h2 = Q^T w' from one read of
// the basis (streamed, row-owner form).
//
// The p * C row chunks of 128 rows (probe b, chunk c -> flat index b C + c)
// are cut into one equal contiguous range per resident CTA, so every SM
// streams the same share.  A CTA walks its range through a ring of nbuf
// shared-memory buffers filled by a copy warp: 2-D tensor copies of 128 rows
// x 8 basis vectors, 1-D copies for a tail of fewer than 8 vectors and for
// the chunk's rows of w, all completing on the buffer's "full" barrier; the
// four row warps release a buffer through its "empty" barrier.  Thread j
// owns row j of every chunk:
//   w'[j] = w[j] - sum_i q_i[j] c_i           (its own row only)
//   h2_i += q_i[j] w'[j]   for every i        (a register per vector)
// so no data crosses threads until the CTA leaves a probe, when the
// per-thread float sums (one product per chunk) go through a warp butterfly
// and a fixed-order float64 sum over warps.  A probe split between CTAs is
// finished by the last of them to arrive, summing their partials in CTA
// order, so results do not depend on timing.  Vectors are padded to a
// multiple of 8 with zero columns that no copy writes.
// ---------------------------------------------------------------------------

// Bounded, sleeping wait for the phase of `bar` with the given parity.
__device__ __forceinline__ bool bar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                 volatile int *fail,
                                                 uint64_t limit_ns = kMbarWaitNs) {
  return mbar_wait_bounded(smem_addr(bar), parity, fail, limit_ns);
}

constexpr int kSThreads = 128;
constexpr int kSWarps = kSThreads / 32;
constexpr int kSR = 128;
constexpr int kSMaxBuf = 8;
constexpr int kSMaxGroups = 16;  // ncols <= 128

// Per-thread sums of N values -> per-warp sums: a halving butterfly (each
// step a lane keeps half of its values and adds its partner's copy of that
// half), so N values cost N - N/32 shuffles instead of 5 N.  Afterwards lane
// `lane` holds in v[i], i < max(N / 32, 1), the warp sum of value
// xsum_index<N>(lane, i); for N < 32 lanes with the same index hold copies.
template <int N>
__device__ __forceinline__ int xsum_index(int lane, int i) {
  int idx = i;
#pragma unroll
  for (int s = 0; s < 5; ++s)
    if ((N >> (s + 1)) >= 1 && (lane & (16 >> s))) idx += N >> (s + 1);
  return idx;
}

template <typename T, int N>
__device__ __forceinline__ void warp_xsum(T (&v)[N], int lane) {
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const int o = 16 >> s;
    const int half = N >> (s + 1);
    if (half >= 1) {
      const bool up = (lane & o) != 0;
#pragma unroll
      for (int i = 0; i < half; ++i) {
        const T send = up ? v[i] : v[i + half];
        const T keep = up ? v[i + half] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
    } else {
      v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
    }
  }
}

__device__ __forceinline__ void row_warps_sync() {
  asm volatile("bar.sync 1, %0;" ::"n"(kSThreads) : "memory");
}

// The flat chunk sequence f = b * C + c (probe b, chunk c of C) is cut into
// gridDim.x equal ranges; range x is [F x / G, F (x + 1) / G).  The CTA that
// covers flat chunk f:
__device__ __forceinline__ int64_t cta_of_chunk(int64_t f, int64_t F, int64_t G) {
  return ((f + 1) * G - 1) / F;
}

// What one pass of the streamed kernel computes per probe:
//   kStreamSubProj  w' = w - Q c (stored), h_i = q_i . w'      (second CGS2 pass)
//   kStreamProj     h_i = q_i . w                              (first CGS2 pass)
//   kStreamSubNorm  w' = w - Q c (stored), ||w'||              (final CGS2 update)
// and, for the two-sweep Arnoldi step, with two vectors per probe (a = w,
// b = the second vector):
//   kStreamProj2    h_i = q_i . b, g_i = q_i . a, a . b
//   kStreamSub2     b' = b - Q h (stored in a third array), a' = a - Q g
//                   (stored over a), ||b'||^2, ||a'||^2, b' . a'
enum : int { kStreamSubProj = 0, kStreamProj = 1, kStreamSubNorm = 2, kStreamProj2 = 3, kStreamSub2 = 4 };

// Per-probe outputs of a pass (the cross-CTA partial-sum stride).
template <int MAXG, int kMode>
__host__ __device__ constexpr int stream_nout_max() {
  return kMode == kStreamProj2 ? 2 * kSPGroup * MAXG + 1
                               : (kMode == kStreamSub2 ? 3 : (kMode == kStreamSubNorm ? 1 : kSPGroup * MAXG));
}

// kRPT: rows of a chunk per row thread (chunks of kSR * kRPT rows).  Chunks
// of few vectors are small, and a pass over them is bound by the number of
// bulk copies and per-chunk steps rather than by bytes; the two-sweep modes
// with at most 8 vectors take 4 rows a thread (2 KB copies, 1-D only).
template <typename T, int MAXG, bool kHold, int kMode, int kRPT = 1>
__global__ void __launch_bounds__(kSThreads + 32)
stream_sweep_kernel(const __grid_constant__ CUtensorMap qmap, const T *__restrict__ Q,
                    int64_t q_bstride, int64_t q_istride, int ncols,
                    const double *__restrict__ coef, int64_t c_bstride, int64_t c_istride,
                    T *Wv, int64_t w_bstride, const T *Wv2, int64_t w2_bstride, T *Wo2,
                    int64_t wo2_bstride, int64_t koff, int coff, int64_t n, int64_t p, int nbuf,
                    int pstride,
                    double *__restrict__ partials, unsigned *__restrict__ counters,
                    double *__restrict__ out, int64_t out_bstride, int64_t out_istride,
                    double *__restrict__ out2, int64_t out2_bstride, int *__restrict__ status) {
  constexpr bool kPair = kMode == kStreamProj2 || kMode == kStreamSub2;  // two vectors a probe
  constexpr bool kUpdate = kMode == kStreamSubProj || kMode == kStreamSubNorm || kMode == kStreamSub2;
  constexpr bool kDots = kMode == kStreamSubProj || kMode == kStreamProj || kMode == kStreamProj2;
  constexpr int kNV = kPair ? 2 : 1;
  constexpr int kNAcc = kDots ? kSPGroup * MAXG : 1;
  static_assert(kRPT == 1 || !kHold, "register-held basis values are for one row a thread");
  constexpr int CR = kSR * kRPT;  // rows of a chunk
  extern __shared__ __align__(128) uint8_t smem[];
  const int ngroups = (ncols + kSPGroup - 1) / kSPGroup;
  const int cpad = ngroups * kSPGroup;
  const int nout = kMode == kStreamProj2 || kMode == kStreamSub2 ? stream_nout_max<MAXG, kMode>()
                                                                 : (kDots ? ncols : 1);
  // ring of nbuf buffers [cpad + kNV][CR]: the chunk's basis rows (zero
  // columns past ncols), then its rows of w (and of the second vector)
  T *bufs = reinterpret_cast<T *>(smem);
  const size_t bstr = (size_t)(cpad + kNV) * CR;
  T *s_coef = bufs + nbuf * bstr;  // [kNV][cpad], zero past ncols
  __shared__ __align__(8) uint64_t full_bar[kSMaxBuf];   // copies of the chunk landed
  __shared__ __align__(8) uint64_t empty_bar[kSMaxBuf];  // every row warp is done with it
  __shared__ double red[kSWarps][kSPGroup * kSMaxGroups + 1];
  __shared__ int s_fail;
  __shared__ int s_last;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t C = (n + CR - 1) / CR;
  const int64_t F = p * C;
  const int64_t G = gridDim.x;
  const int64_t f_begin = F * (int64_t)blockIdx.x / G;
  const int64_t f_end = F * ((int64_t)blockIdx.x + 1) / G;
  const int kcols = (int)(q_bstride / q_istride);

  if (threadIdx.x == 0) {
    for (int u = 0; u < nbuf; ++u) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&full_bar[u])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&empty_bar[u])),
                   "r"(kSWarps)
                   : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_fail = 0;
  }
  if (threadIdx.x < kSR)
    for (int u = 0; u < nbuf; ++u)
      for (int i = ncols; i < cpad; ++i)
#pragma unroll
        for (int rr = 0; rr < kRPT; ++rr) bufs[u * bstr + (size_t)i * CR + rr * kSR + threadIdx.x] = (T)0;
  // 2-D tensor copies need a 128-byte aligned shared destination; if the
  // ring is not aligned, record it and load every vector with 1-D copies
  const bool tile_ok = (smem_addr(bufs) & 127u) == 0;
  if (!tile_ok && threadIdx.x == 0 && status) atomicExch(status, (int)MFG_ERR_BAD_ARG);
  // (2-D boxes are kSR rows high: chunks of several rows a thread use 1-D copies)
  const int full = (tile_ok && kRPT == 1) ? ncols / kSPGroup : 0;
  __syncthreads();
  volatile int *fail = &s_fail;

  if (warp == kSWarps) {
    // copy warp: chunk t of this CTA goes into buffer t % nbuf once the row
    // warps have released that buffer's previous chunk; lane cp issues
    // copies cp, cp + 32, ... of a chunk
    int issued = 0;
    const int ncopies = full + (ncols - full * kSPGroup) + kNV;
    // position of chunk t: probe b, row chunk c, buffer u used for the
    // (ph)-parity time; advanced without divisions
    int64_t b = f_begin / C, c = f_begin - (f_begin / C) * C;
    int u = 0;
    uint32_t ph = 0;
    const int nt = (int)(f_end - f_begin);
    for (int t = 0; t < nt; ++t) {
      if (t >= nbuf && !bar_wait_bounded(&empty_bar[u], ph ^ 1u, fail)) {
        if (lane == 0) {
          *fail = 1;
          if (status) atomicExch(status, (int)MFG_ERR_TIMEOUT);
        }
        break;
      }
      const int64_t r0 = c * CR;
      const int64_t rows = (n - r0 < CR) ? (n - r0) : CR;
      const uint32_t seg_bytes = (uint32_t)(((rows * (int64_t)sizeof(T)) + 15) / 16 * 16);
      const uint32_t bytes = (uint32_t)full * (uint32_t)(kSPGroup * kSR * sizeof(T)) +
                             seg_bytes * (uint32_t)(ncols - full * kSPGroup + kNV);
      if (lane == 0)
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                         smem_addr(&full_bar[u])),
                     "r"(bytes)
                     : "memory");
      __syncwarp();
      T *dst = bufs + u * bstr;
      for (int cp = lane; cp < ncopies; cp += 32) {
        if (cp < full) {
          const int x = (int)r0, y = (int)(b * kcols + coff + cp * kSPGroup);
          asm volatile(
              "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
              "[%0], [%1, {%3, %4}], [%2];" ::"r"(smem_addr(dst + (size_t)cp * kSPGroup * kSR)),
              "l"(reinterpret_cast<uint64_t>(&qmap)), "r"(smem_addr(&full_bar[u])), "r"(x), "r"(y)
              : "memory");
        } else {
          // a tail vector, or (last kNV copies) the chunk's rows of w and of
          // the second vector
          const int i = full * kSPGroup + (cp - full);
          const int vec = cp - (ncopies - kNV);  // 0: w, 1: second vector, < 0: basis
          const T *src = vec == 0   ? Wv + b * w_bstride + r0
                         : vec == 1 ? Wv2 + b * w2_bstride + r0
                                    : Q + b * q_bstride + (int64_t)(coff + i) * q_istride + r0;
          T *d = dst + (size_t)(vec >= 0 ? cpad + vec : i) * CR;
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
              ::"r"(smem_addr(d)), "l"(reinterpret_cast<uint64_t>(src)), "r"(seg_bytes),
              "r"(smem_addr(&full_bar[u]))
              : "memory");
        }
      }
      issued = t + 1;
      if (++c == C) {
        c = 0;
        ++b;
      }
      if (++u == nbuf) {
        u = 0;
        ph ^= 1u;
      }
    }
    if (*fail && lane == 0) {
      // the copies of the last chunks issued land (bounded) before the CTA's
      // shared memory goes away; earlier buffers were consumed before reuse
      for (int t = (issued > nbuf ? issued - nbuf : 0); t < issued; ++t)
        bar_wait_bounded(&full_bar[t % nbuf], (uint32_t)((t / nbuf) & 1), nullptr, kMbarWaitNs / 8);
    }
  } else {
    // row warps: thread j owns row j of every chunk
    const int j = threadIdx.x;
    T acc[kNAcc];
    T accg[kMode == kStreamProj2 ? kNAcc : 1];  // kStreamProj2: q_i . w (acc: q_i . b)
#pragma unroll
    for (int i = 0; i < kNAcc; ++i) acc[i] = (T)0;
#pragma unroll
    for (int i = 0; i < (kMode == kStreamProj2 ? kNAcc : 1); ++i) accg[i] = (T)0;
    T cross = (T)0;    // a . b over this thread's rows (kStreamProj2)
    double nrm = 0.0;  // ||w'||^2 over this thread's rows (kStreamSubNorm, kStreamSub2: ||b'||^2)
    double nrm2 = 0.0, dot2 = 0.0;  // kStreamSub2: ||a'||^2, b' . a'
    int64_t b = f_begin / C, c = f_begin - (f_begin / C) * C;
    int u = 0;
    uint32_t ph = 0;
    const int nt = (int)(f_end - f_begin);
    for (int t = 0; t < nt; ++t) {
      if (t == 0 || c == 0) {
        if constexpr (kUpdate) {
          // a new probe: its coefficients (the row warps are past every read
          // of the previous ones)
          row_warps_sync();
          for (int i = j; i < cpad; i += kSThreads) {
            s_coef[i] = i < ncols ? (T)coef[b * c_bstride + i * c_istride] : (T)0;
            if constexpr (kPair) s_coef[cpad + i] = i < ncols ? (T)coef[b * c_bstride + koff + i] : (T)0;
          }
          row_warps_sync();
        }
      }
      // After a failure every row warp still walks the remaining chunks
      // (without waiting or computing), so all of them meet at the same
      // named barriers.
      bool ready = false;
      if (!*fail) {
        ready = bar_wait_bounded(&full_bar[u], ph, fail);
        if (!ready) {
          *fail = 1;
          if (status) atomicExch(status, (int)MFG_ERR_TIMEOUT);
        }
      }
      const int64_t r0 = c * CR;
      const int rows = (int)((n - r0 < CR) ? (n - r0) : CR);
#pragma unroll
      for (int rr = 0; rr < kRPT; ++rr) {
        const int jr = j + rr * kSR;            // this thread's row of the chunk
        const T *buf = bufs + u * bstr + jr;  // column stride CR
        T qv[kHold ? kSPGroup * MAXG : 1];
        T w = ready ? buf[(size_t)cpad * CR] : (T)0;
        T w2v = (kPair && ready) ? buf[(size_t)(cpad + 1) * CR] : (T)0;  // second vector
        if constexpr (kMode == kStreamSub2) {
          // b' = b - Q h and a' = a - Q g over this thread's row
          T a0 = w, a1 = (T)0, b0 = w2v, b1 = (T)0;
#pragma unroll
          for (int g = 0; g < MAXG; ++g)
            if (ready && g < ngroups) {
#pragma unroll
              for (int e = 0; e < kSPGroup; e += 2) {
                const int i = g * kSPGroup + e;
                const T q0 = buf[(size_t)i * CR], q1 = buf[(size_t)(i + 1) * CR];
                b0 = fma(-q0, s_coef[i], b0);
                b1 = fma(-q1, s_coef[i + 1], b1);
                a0 = fma(-q0, s_coef[cpad + i], a0);
                a1 = fma(-q1, s_coef[cpad + i + 1], a1);
              }
            }
          w = a0 + a1;
          w2v = b0 + b1;
        } else if constexpr (kUpdate) {
          // w' = w - Q c over this thread's row; four interleaved sums shorten
          // the dependent chain
          T w0 = w, w1 = (T)0, w2 = (T)0, w3 = (T)0;
#pragma unroll
          for (int g = 0; g < MAXG; ++g)
            if (ready && g < ngroups) {
#pragma unroll
              for (int e = 0; e < kSPGroup; e += 4) {
                const int i = g * kSPGroup + e;
                const T q0 = buf[(size_t)i * CR], q1 = buf[(size_t)(i + 1) * CR];
                const T q2 = buf[(size_t)(i + 2) * CR], q3 = buf[(size_t)(i + 3) * CR];
                if constexpr (kHold) {
                  qv[i] = q0;
                  qv[i + 1] = q1;
                  qv[i + 2] = q2;
                  qv[i + 3] = q3;
                }
                w0 = fma(-q0, s_coef[i], w0);
                w1 = fma(-q1, s_coef[i + 1], w1);
                w2 = fma(-q2, s_coef[i + 2], w2);
                w3 = fma(-q3, s_coef[i + 3], w3);
              }
            }
          w = (w0 + w1) + (w2 + w3);
        }
        // rows past the probe's end hold stale shared memory and are left out
        if (ready && jr < rows) {
          if constexpr (kUpdate) Wv[b * w_bstride + r0 + jr] = w;
          if constexpr (kMode == kStreamSubNorm) {
            const T w2 = w * w;
            nrm += (double)w2;
          }
          if constexpr (kMode == kStreamSub2) {
            Wo2[b * wo2_bstride + r0 + jr] = w2v;
            nrm += (double)(w2v * w2v);
            nrm2 += (double)(w * w);
            dot2 += (double)(w2v * w);
          }
          if constexpr (kMode == kStreamProj2) {
#pragma unroll
            for (int g = 0; g < MAXG; ++g)
              if (g < ngroups) {
#pragma unroll
                for (int e = 0; e < kSPGroup; ++e) {
                  const int i = g * kSPGroup + e;
                  const T q = buf[(size_t)i * CR];
                  acc[i] = fma(q, w2v, acc[i]);
                  accg[i] = fma(q, w, accg[i]);
                }
              }
            cross = fma(w, w2v, cross);
          } else if constexpr (kDots) {
#pragma unroll
            for (int g = 0; g < MAXG; ++g)
              if (g < ngroups) {
#pragma unroll
                for (int e = 0; e < kSPGroup; ++e) {
                  const int i = g * kSPGroup + e;
                  const T q = kHold ? qv[kHold ? i : 0] : buf[(size_t)i * CR];
                  acc[i] = fma(q, w, acc[i]);
                }
              }
          }
        }
      }
      __syncwarp();
      if (lane == 0 && ready)
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(&empty_bar[u])) : "memory");

      // the probe's last row chunk in this CTA: its share of the outputs
      if (t + 1 == nt || c + 1 == C) {
        if constexpr (kDots) {
          // per-thread float sums -> warp butterfly -> fixed-order warp sum
          warp_xsum<T, kNAcc>(acc, lane);
          constexpr int kPer = kNAcc / 32 > 0 ? kNAcc / 32 : 1;
          constexpr int kDup = kNAcc >= 32 ? 1 : 32 / kNAcc;
          if ((lane & (kDup - 1)) == 0) {
#pragma unroll
            for (int i = 0; i < kPer; ++i) red[warp][xsum_index<kNAcc>(lane, i)] = (double)acc[i];
          }
#pragma unroll
          for (int i = 0; i < kNAcc; ++i) acc[i] = (T)0;
          if constexpr (kMode == kStreamProj2) {
            // second half of the outputs: q_i . w, then a . b
            warp_xsum<T, kNAcc>(accg, lane);
            if ((lane & (kDup - 1)) == 0) {
#pragma unroll
              for (int i = 0; i < kPer; ++i) red[warp][kNAcc + xsum_index<kNAcc>(lane, i)] = (double)accg[i];
            }
#pragma unroll
            for (int i = 0; i < kNAcc; ++i) accg[i] = (T)0;
            const double v = warp_sum((double)cross);
            if (lane == 0) red[warp][2 * kNAcc] = v;
            cross = (T)0;
          }
        } else if constexpr (kMode == kStreamSub2) {
          const double v0 = warp_sum(nrm), v1 = warp_sum(nrm2), v2 = warp_sum(dot2);
          if (lane == 0) {
            red[warp][0] = v0;
            red[warp][1] = v1;
            red[warp][2] = v2;
          }
          nrm = nrm2 = dot2 = 0.0;
        } else {
          const double v = warp_sum(nrm);
          if (lane == 0) red[warp][0] = v;
          nrm = 0.0;
        }
        row_warps_sync();
        // thread j reduces outputs j and j + kSThreads (at most nout <= 2 kSThreads + 1)
        constexpr int kOut = kMode == kStreamProj2 ? 2 : 1;
        double h[kOut];
#pragma unroll
        for (int o = 0; o < kOut; ++o) {
          const int v = j + o * kSThreads;
          h[o] = 0.0;
          if (v < nout) {
#pragma unroll
            for (int q = 0; q < kSWarps; ++q) h[o] += red[q][v];
          }
        }
        const int64_t first = cta_of_chunk(b * C, F, G), last = cta_of_chunk(b * C + C - 1, F, G);
        bool emit = first == last;
        if (!emit) {
          const int64_t seg = (int64_t)blockIdx.x - first;
#pragma unroll
          for (int o = 0; o < kOut; ++o) {
            const int v = j + o * kSThreads;
            if (v < nout) partials[(b * pstride + seg) * nout + v] = h[o];
          }
          __threadfence();
          row_warps_sync();
          if (j == 0) {
            const unsigned ticket = atomicAdd(&counters[b], 1u);
            s_last = ticket == (unsigned)(last - first);
          }
          row_warps_sync();
          if (s_last) {
            __threadfence();
            emit = true;
#pragma unroll
            for (int o = 0; o < kOut; ++o) {
              const int v = j + o * kSThreads;
              if (v < nout) {
                h[o] = 0.0;
                for (int64_t q = 0; q <= last - first; ++q)
                  h[o] += __ldcg(&partials[(b * pstride + q) * nout + v]);
              }
            }
            if (j == 0) counters[b] = 0u;
          }
        }
        if (emit) {
#pragma unroll
          for (int o = 0; o < kOut; ++o) {
            const int v = j + o * kSThreads;
            if (v >= nout) continue;
            if constexpr (kMode == kStreamSubNorm) {
              const double nv = sqrt(h[o]);
              if (out) out[b * out_bstride] = nv;
              if (out2) out2[b * out2_bstride] = nv;
            } else if constexpr (kMode == kStreamSub2) {
              out[b * out_bstride + v] = h[o];
            } else if constexpr (kMode == kStreamProj2) {
              constexpr int kHalf = kSPGroup * MAXG;
              if (v == 2 * kHalf) {
                if (out2)
                  out2[b * out2_bstride] = h[o];
                else
                  out[b * out_bstride + 2 * koff] = h[o];
              } else {
                const int half = v / kHalf, i = v - half * kHalf;
                if (i < ncols) out[b * out_bstride + half * koff + i] = h[o];
              }
            } else {
              out[b * out_bstride + v * out_istride] = h[o];
            }
          }
        }
        // red and s_last are reused at this CTA's next probe
        row_warps_sync();
      }
      if (++c == C) {
        c = 0;
        ++b;
      }
      if (++u == nbuf) {
        u = 0;
        ph ^= 1u;
      }
    }
  }
  __syncthreads();
}

template <typename T>
static size_t stream_sweep_smem(int ncols, int nbuf, int nv = 1, int rpt = 1) {
  const int cpad = (ncols + kSPGroup - 1) / kSPGroup * kSPGroup;
  return (size_t)nbuf * (cpad + nv) * kSR * rpt * sizeof(T) + (size_t)nv * cpad * sizeof(T);
}

// Largest vector count of the streamed sweeps: 128 floats, 64 doubles (the
// per-thread dot-product sums live in registers).
template <typename T> constexpr int stream_sweep_max_cols() { return sizeof(T) == 4 ? 128 : 64; }

// Ring depth: as many buffers (2..8) as fit in ~110 KB, so that two CTAs
// share an SM; 0 if the sweep does not apply.
template <typename T>
static int stream_sweep_buffers(int ncols, int nv = 1, int rpt = 1) {
  if (ncols < 1 || ncols > stream_sweep_max_cols<T>()) return 0;
  int nb = kSMaxBuf;
  while (nb > 2 && stream_sweep_smem<T>(ncols, nb, nv, rpt) > 110 * 1024) --nb;
  return stream_sweep_smem<T>(ncols, nb, nv, rpt) <= 220 * 1024 ? nb : 0;
}

struct StreamArgs {
  const void *Q;
  int64_t q_bstride, q_istride;
  int ncols;
  const double *coef;
  int64_t c_bstride, c_istride;
  void *Wv;
  int64_t w_bstride, n, p;
  double *partials;
  unsigned *counters;
  double *out;
  int64_t out_bstride, out_istride;
  double *out2;
  int64_t out2_bstride;
  int *status;
  // two-vector passes: the second vector, where its update goes, and the
  // offset of the second coefficient / output block of a probe
  const void *Wv2 = nullptr;
  int64_t w2_bstride = 0;
  void *Wo2 = nullptr;
  int64_t wo2_bstride = 0, koff = 0;
  int coff = 0;  // first basis vector of the pass (the vectors are coff .. coff + ncols - 1)
};

template <typename T, int MAXG, bool kHold, int kMode, int kRPT = 1>
static int launch_stream_sweep_t(const StreamArgs &a, cudaStream_t s) {
  constexpr int nv = (kMode == kStreamProj2 || kMode == kStreamSub2) ? 2 : 1;
  const int nbuf = stream_sweep_buffers<T>(a.ncols, nv, kRPT);
  if (nbuf < 2) return MFG_ERR_UNSUPPORTED;
  const size_t smem = stream_sweep_smem<T>(a.ncols, nbuf, nv, kRPT);
  if (a.q_istride <= 0 || a.q_bstride % a.q_istride != 0) return MFG_ERR_BAD_ARG;
  auto kern = stream_sweep_kernel<T, MAXG, kHold, kMode, kRPT>;
  // The default dynamic limit is 48 KB minus the kernel's static shared
  // memory, so the opt-in is raised well below 48 KB.
  if (smem > 32 * 1024)
    MFG_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // resident CTAs per SM for this vector count (cached: the answer depends
  // only on the shared-memory size, i.e. on ncols)
  static int per_sm_cache[129];  // one cache per template instance
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    MFG_CUDA_TRY(cudaGetDevice(&dev));
    MFG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  }
  int per_sm = per_sm_cache[a.ncols];
  if (per_sm == 0) {
    MFG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSThreads + 32, smem));
    if (per_sm < 1) return MFG_ERR_UNSUPPORTED;
    per_sm_cache[a.ncols] = per_sm;
  }
  // One wave of CTAs, each with an equal share of the p * C row chunks.  A
  // probe then spans at most ceil(G / p) + 1 CTAs, whose partial sums must
  // fit the workspace's max_fused_chunks(n) slots per probe.
  const int64_t C = ceil_div(a.n, (int64_t)kSR * kRPT);
  const int64_t F = a.p * C;
  const int64_t cap = max_fused_chunks<T>(a.n);
  int64_t G = (int64_t)sms * per_sm;
  if (G > F) G = F;
  if (G > a.p * (cap - 1)) G = a.p * (cap - 1);
  if (G < 1) G = 1;
  const int pstride = (int)(ceil_div(G, a.p) + 1);
  // the basis as rows of q_istride elements: row b * k + i is probe b's
  // vector i (only read through 2-D copies when there are 8 or more vectors)
  CUtensorMap qmap;
  memset(&qmap, 0, sizeof(qmap));
  const int64_t kcols = a.q_bstride / a.q_istride;
  if (a.ncols >= kSPGroup &&
      !make_plain_tensor_map_2d(&qmap, (int)sizeof(T), a.Q, a.n, a.p * kcols, a.q_istride,
                                (uint32_t)kSR, (uint32_t)kSPGroup))
    return MFG_ERR_CUDA;
  kern<<<(unsigned)G, kSThreads + 32, smem, s>>>(
      qmap, static_cast<const T *>(a.Q), a.q_bstride, a.q_istride, a.ncols, a.coef, a.c_bstride,
      a.c_istride, static_cast<T *>(a.Wv), a.w_bstride, static_cast<const T *>(a.Wv2),
      a.w2_bstride, static_cast<T *>(a.Wo2), a.wo2_bstride, a.koff, a.coff, a.n, a.p, nbuf, pstride,
      a.partials, a.counters, a.out, a.out_bstride, a.out_istride, a.out2, a.out2_bstride,
      a.status);
  return MFG_LAUNCH_STATUS();
}

template <typename T, int kMode>
static int launch_stream_sweep(const StreamArgs &a, cudaStream_t s) {
  if constexpr (kMode == kStreamProj2 || kMode == kStreamSub2) {
    // two vectors: float bases of up to 64 vectors (the per-thread sums of
    // both vectors stay in registers), no register-held basis values
    if constexpr (sizeof(T) != 4) {
      return MFG_ERR_UNSUPPORTED;
    } else {
      if (a.ncols < 1 || a.ncols > kTwoSweepPassCols) return MFG_ERR_UNSUPPORTED;
      if (a.ncols <= 8) return launch_stream_sweep_t<T, 1, false, kMode, 4>(a, s);
      if (a.ncols <= 32) return launch_stream_sweep_t<T, 4, false, kMode>(a, s);
      return launch_stream_sweep_t<T, 8, false, kMode>(a, s);
    }
  }
  if (stream_sweep_buffers<T>(a.ncols) == 0) return MFG_ERR_UNSUPPORTED;
  // loops (and, for dot products, register sums) sized to the vector count:
  // 8, 32, 64 or 128; in the two-pass form up to 64 (32 doubles) basis
  // values also stay in registers between the passes
  constexpr bool kTwo = kMode == kStreamSubProj;
  if (a.ncols <= 8) return launch_stream_sweep_t<T, 1, kTwo, kMode>(a, s);
  if (a.ncols <= 32) return launch_stream_sweep_t<T, 4, kTwo, kMode>(a, s);
  if (a.ncols <= 64) return launch_stream_sweep_t<T, 8, kTwo && sizeof(T) == 4, kMode>(a, s);
  if constexpr (sizeof(T) == 4) return launch_stream_sweep_t<T, 16, false, kMode>(a, s);
  return MFG_ERR_UNSUPPORTED;
}

// 1 when the fused update+projection applies to this vector count, else 0.
template <typename T>
int sub_proj_rows_per_thread(int ncols) {
  return stream_sweep_buffers<T>(ncols) > 0 ? 1 : 0;
}

// Partial-sum slots per probe of the cross-CTA reductions (at least 2: the
// streamed update+projection splits a probe between up to ceil(G / p) + 1 CTAs).
template <typename T> int64_t max_fused_chunks(int64_t n) {
  const int64_t c = ceil_div(n, kThreads);
  return c < 2 ? 2 : c;
}

template <typename T>
int launch_sub_proj(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols, const double *coef,
                    int64_t c_bstride, int64_t c_istride, T *Wv, int64_t w_bstride, int64_t n,
                    int64_t p, double *partials, unsigned *counters, double *out,
                    int64_t out_bstride, int *status, cudaStream_t s) {
  if (ncols <= 0 || p <= 0) return MFG_OK;
  const StreamArgs a{Q,        q_bstride, q_istride, ncols, coef, c_bstride,   c_istride,
                     Wv,       w_bstride, n,         p,     partials, counters, out,
                     out_bstride, 1,      nullptr,   0,     status};
  return launch_stream_sweep<T, kStreamSubProj>(a, s);
}

template <typename T>
int launch_proj(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols, const T *Wv,
                int64_t w_bstride, int64_t n, int64_t p, double *partials, unsigned *counters,
                double *out, int64_t out_bstride, int64_t out_istride, cudaStream_t s,
                int *status) {
  if (ncols <= 0 || p <= 0) return MFG_OK;
  // the streamed sweep pays a fixed cost per launch that only pays off over
  // enough row chunks (e.g. not for one CG vector of 8192 rows)
  if (stream_sweep_buffers<T>(ncols) > 0 && p * ceil_div(n, (int64_t)kSR) >= 256) {
    const StreamArgs a{Q,        q_bstride, q_istride,   ncols,       nullptr, 0,   0,
                       const_cast<T *>(Wv), w_bstride,   n,           p,       partials,
                       counters, out,       out_bstride, out_istride, nullptr, 0,   status};
    return launch_stream_sweep<T, kStreamProj>(a, s);
  }
  const int64_t nch = num_chunks<T>(n);
  if (p > 65535 || ncols > kMaxProjCols) return MFG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)nch, (unsigned)p);
  const size_t smem = (size_t)ncols * kWarps * sizeof(double);
  proj_kernel<T><<<grid, kThreads, smem, s>>>(Q, q_bstride, q_istride, ncols, Wv, w_bstride, n,
                                              (int)nch, partials, counters, out, out_bstride,
                                              out_istride);
  return MFG_LAUNCH_STATUS();
}

template <typename T>
int launch_sub(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols, const double *coef,
               int64_t c_bstride, int64_t c_istride, const T *Win, T *Wout, int64_t w_bstride,
               int64_t n, int64_t p, bool with_norm, bool store, double *partials,
               unsigned *counters, double *norm_out, double *norm_out2, int64_t norm2_bstride,
               cudaStream_t s, int *status) {
  if (p <= 0) return MFG_OK;
  // in-place updates with a norm go through the streamed sweep; measured on
  // the adjoint, updates without one are faster on the chunked kernel
  if (with_norm && store && Win == Wout && ncols > 0 && stream_sweep_buffers<T>(ncols) > 0) {
    const StreamArgs a{Q,        q_bstride, q_istride, ncols,   coef,      c_bstride,    c_istride,
                       Wout,     w_bstride, n,         p,       partials,  counters,     norm_out,
                       1,        0,         norm_out2, norm2_bstride, status};
    return launch_stream_sweep<T, kStreamSubNorm>(a, s);
  }
  const int64_t nch = num_chunks<T>(n);
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)nch, (unsigned)p);
  const size_t smem = (size_t)(ncols > 0 ? ncols : 1) * sizeof(T);
  if (smem > 40 * 1024) return MFG_ERR_UNSUPPORTED;  // under the default dynamic limit
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
  return MFG_LAUNCH_STATUS();
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
  return MFG_LAUNCH_STATUS();
}

int launch_inv(const double *x, double *y, int64_t p, cudaStream_t s) {
  if (p <= 0) return MFG_OK;
  inv_kernel<<<(unsigned)ceil_div(p, 128), 128, 0, s>>>(x, y, p);
  return MFG_LAUNCH_STATUS();
}

// ---------------------------------------------------------------------------
// Conjugate gradients, one independent CG per probe row of a panel (as
// jax.scipy.sparse.linalg.cg under vmap: a finished probe stays frozen while
// the others iterate).  The vector updates of an iteration carry the float64
// squared norm of the new residual, summed across CTAs in chunk order.
// ---------------------------------------------------------------------------

// CTA sum of a per-thread float64 value, then the cross-CTA sum of probe b
// in chunk order by the last CTA to arrive; returns true (with *total) in
// that CTA's thread 0.
__device__ __forceinline__ bool probe_sum(double v, int64_t b, int64_t c, int nchunks,
                                          double *partials, unsigned *counters, double *total) {
  __shared__ double red[kWarps];
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < kWarps; ++q) t += red[q];
    if (nchunks == 1) {
      *total = t;
      return true;
    }
    partials[b * nchunks + c] = t;
  }
  if (nchunks == 1) return false;
  if (!arrive_last(counters, b, nchunks)) return false;
  if (threadIdx.x != 0) return false;
  t = 0.0;
  for (int q = 0; q < nchunks; ++q) t += __ldcg(&partials[b * nchunks + q]);
  counters[b] = 0u;
  *total = t;
  return true;
}

template <typename T>
__device__ __forceinline__ void store_split(const T (&w)[kVPT][Vec<T>::width], int64_t n, int64_t c,
                                            __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
  constexpr int W = Vec<T>::width;
#pragma unroll
  for (int e = 0; e < kVPT; ++e) {
    const int64_t r = c * chunk_rows<T>() + ((int64_t)e * kThreads + threadIdx.x) * W;
    if (r >= n) continue;
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const float x = (float)w[e][u];
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      hi[r + u] = h;
      if (lo) lo[r + u] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
  }
}

// X = 0, R = P = B, rs = ||B||^2, thr = max(tol^2 ||B||^2, atol^2)
template <typename T>
__global__ void __launch_bounds__(kThreads)
cg_init_kernel(const T *__restrict__ B, T *__restrict__ X, T *__restrict__ R, T *__restrict__ P,
               int64_t ld, int64_t n, __nv_bfloat16 *hi, __nv_bfloat16 *lo, int nchunks,
               double *partials, unsigned *counters, double tol2, double atol2,
               double *__restrict__ rs, double *__restrict__ thr, int *__restrict__ iters) {
  constexpr int W = Vec<T>::width;
  const int64_t c = blockIdx.x, b = blockIdx.y;
  T w[kVPT][W], z[kVPT][W];
  load_chunk<T>(B + b * ld, n, c, w);
  double acc = 0.0;
#pragma unroll
  for (int e = 0; e < kVPT; ++e)
#pragma unroll
    for (int u = 0; u < W; ++u) {
      acc = fma((double)w[e][u], (double)w[e][u], acc);
      z[e][u] = (T)0;
    }
  store_chunk<T>(X + b * ld, n, c, z);
  store_chunk<T>(R + b * ld, n, c, w);
  store_chunk<T>(P + b * ld, n, c, w);
  if (hi) store_split<T>(w, n, c, hi + b * ld, lo ? lo + b * ld : nullptr);
  double t;
  if (probe_sum(acc, b, c, nchunks, partials, counters, &t)) {
    rs[b] = t;
    thr[b] = fmax(tol2 * t, atol2);
    if (iters) iters[b] = 0;
  }
}

// For a probe still running (rs > thr): alpha = rs / pAp, X += alpha P,
// R -= alpha W; every probe: rs_next = ||R||^2.  The last CTA of a probe
// counts it into *nactive when it keeps running after this iteration; the
// count alternates between two slots, and this launch zeroes the slot of the
// next iteration (*nactive_clear).
template <typename T>
__global__ void __launch_bounds__(kThreads)
cg_update_kernel(T *__restrict__ X, T *__restrict__ R, const T *__restrict__ P,
                 const T *__restrict__ W, int64_t ld, int64_t n, const double *__restrict__ rs,
                 const double *__restrict__ pap, const double *__restrict__ thr, int nchunks,
                 double *partials, unsigned *counters, double *__restrict__ rs_next,
                 int *__restrict__ nactive, int *__restrict__ nactive_clear,
                 int *__restrict__ iters) {
  constexpr int VW = Vec<T>::width;
  const int64_t c = blockIdx.x, b = blockIdx.y;
  if (c == 0 && b == 0 && threadIdx.x == 0) *nactive_clear = 0;  // the next iteration's count
  const bool active = rs[b] > thr[b];
  T r[kVPT][VW];
  load_chunk<T, false>(R + b * ld, n, c, r);
  if (active) {
    __shared__ T alpha_s;  // one float64 division per CTA, not per thread
    if (threadIdx.x == 0) alpha_s = (T)(rs[b] / pap[b]);
    __syncthreads();
    const T alpha = alpha_s;
    T x[kVPT][VW], pv[kVPT][VW], wv[kVPT][VW];
    load_chunk<T, false>(X + b * ld, n, c, x);
    load_chunk<T>(P + b * ld, n, c, pv);
    load_chunk<T>(W + b * ld, n, c, wv);
#pragma unroll
    for (int e = 0; e < kVPT; ++e)
#pragma unroll
      for (int u = 0; u < VW; ++u) {
        x[e][u] = fma(alpha, pv[e][u], x[e][u]);
        r[e][u] = fma(-alpha, wv[e][u], r[e][u]);
      }
    store_chunk<T>(X + b * ld, n, c, x);
    store_chunk<T>(R + b * ld, n, c, r);
  }
  double acc = 0.0;
#pragma unroll
  for (int e = 0; e < kVPT; ++e)
#pragma unroll
    for (int u = 0; u < VW; ++u) acc = fma((double)r[e][u], (double)r[e][u], acc);
  double t;
  if (probe_sum(acc, b, c, nchunks, partials, counters, &t)) {
    rs_next[b] = t;
    if (active) {
      if (iters) iters[b] += 1;
      if (t > thr[b]) atomicAdd(nactive, 1);
    }
  }
}

// For a probe that ran this iteration: P = R + (rs_next / rs) P (and its
// bf16 hi / lo copies for the tensor-core operator).
template <typename T>
__global__ void __launch_bounds__(kThreads)
cg_direction_kernel(T *__restrict__ P, const T *__restrict__ R, int64_t ld, int64_t n,
                    const double *__restrict__ rs, const double *__restrict__ rs_next,
                    const double *__restrict__ thr, __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
  constexpr int VW = Vec<T>::width;
  const int64_t c = blockIdx.x, b = blockIdx.y;
  if (!(rs[b] > thr[b])) return;
  __shared__ T beta_s;  // one float64 division per CTA, not per thread
  if (threadIdx.x == 0) beta_s = (T)(rs_next[b] / rs[b]);
  __syncthreads();
  const T beta = beta_s;
  T pv[kVPT][VW], r[kVPT][VW];
  load_chunk<T, false>(P + b * ld, n, c, pv);
  load_chunk<T>(R + b * ld, n, c, r);
#pragma unroll
  for (int e = 0; e < kVPT; ++e)
#pragma unroll
    for (int u = 0; u < VW; ++u) pv[e][u] = fma(beta, pv[e][u], r[e][u]);
  store_chunk<T>(P + b * ld, n, c, pv);
  if (hi) store_split<T>(pv, n, c, hi + b * ld, lo ? lo + b * ld : nullptr);
}

// Short vectors (n <= kCgSmallMaxN): one CTA per probe runs everything of an
// iteration after the operator product -- pAp, X += alpha P, R -= alpha W,
// ||R||^2 and, for a probe that ran, P = R + beta P with its bf16 copies -- in
// one launch, where longer vectors take a projection, an update and a
// direction launch.  Each thread holds its E elements of R, P and W in
// registers (element threadIdx.x + e * 1024), so one round of loads feeds all
// three phases.  The per-element arithmetic is that of cg_update_kernel and
// cg_direction_kernel.  Dot products accumulate in T within a warp and in
// float64 over the 32 warps: this GPU's float64 rate is a small fraction of
// its float32 rate, and one SM doing every product in float64 took longer
// than the three launches it replaces.
constexpr int kCgSmallThreads = 1024;

template <typename T>
__device__ __forceinline__ double cta_sum_small(T v, double *red) {
  v = warp_sum_t<T>(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)v;
  __syncthreads();
  if (threadIdx.x < 32) {
    const double t = warp_sum(red[threadIdx.x]);
    if (threadIdx.x == 0) red[32] = t;
  }
  __syncthreads();
  const double t = red[32];
  __syncthreads();  // red is reused by the next sum
  return t;
}

template <typename T, int E>
__global__ void __launch_bounds__(kCgSmallThreads)
cg_step_small_kernel(T *__restrict__ X, T *__restrict__ R, T *__restrict__ P,
                     const T *__restrict__ W, int64_t ld, int64_t n,
                     const double *__restrict__ rs, const double *__restrict__ thr,
                     double *__restrict__ rs_next, int *__restrict__ nactive,
                     int *__restrict__ nactive_clear, int *__restrict__ iters,
                     __nv_bfloat16 *hi, __nv_bfloat16 *lo) {
  __shared__ double red[33];
  __shared__ T coef;  // alpha, then beta: one float64 division each, in thread 0
  __shared__ int run;
  const int64_t b = blockIdx.x;
  T *x = X + b * ld, *r = R + b * ld, *pv = P + b * ld;
  const T *w = W + b * ld;
  T rv[E], pe[E], we[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {  // issued before the barrier below
    const int i = (int)threadIdx.x + e * kCgSmallThreads;  // n <= kCgSmallMaxN
    const bool in = i < n;
    rv[e] = in ? r[i] : (T)0;
    pe[e] = in ? pv[i] : (T)0;
    we[e] = in ? w[i] : (T)0;
  }
  if (threadIdx.x == 0) {
    if (b == 0) *nactive_clear = 0;  // the next iteration's count
    run = rs[b] > thr[b];
  }
  __syncthreads();
  const bool active = run != 0;  // uniform over the CTA
  T rr = (T)0;
  if (active) {
    T acc = (T)0;
#pragma unroll
    for (int e = 0; e < E; ++e) acc = fma(pe[e], we[e], acc);
    const double pap = cta_sum_small<T>(acc, red);
    if (threadIdx.x == 0) coef = (T)(rs[b] / pap);
    __syncthreads();
    const T alpha = coef;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const int i = (int)threadIdx.x + e * kCgSmallThreads;  // n <= kCgSmallMaxN
      rv[e] = fma(-alpha, we[e], rv[e]);
      if (i < n) {
        x[i] = fma(alpha, pe[e], x[i]);  // X is read only here
        r[i] = rv[e];
      }
    }
  }
#pragma unroll
  for (int e = 0; e < E; ++e) rr = fma(rv[e], rv[e], rr);
  const double t = cta_sum_small<T>(rr, red);  // every thread has read alpha by now
  if (threadIdx.x == 0) {
    rs_next[b] = t;
    if (active) {
      if (iters) iters[b] += 1;
      if (t > thr[b]) atomicAdd(nactive, 1);
      coef = (T)(t / rs[b]);
    }
  }
  if (!active) return;
  __syncthreads();
  const T beta = coef;
  __nv_bfloat16 *h = hi ? hi + b * ld : nullptr, *l = lo ? lo + b * ld : nullptr;
#pragma unroll
  for (int e = 0; e < E; ++e) {
    const int i = (int)threadIdx.x + e * kCgSmallThreads;  // n <= kCgSmallMaxN
    if (i >= n) continue;
    const T pn = fma(beta, pe[e], rv[e]);
    pv[i] = pn;
    if (h) {
      const float f = (float)pn;
      const __nv_bfloat16 hb = __float2bfloat16_rn(f);
      h[i] = hb;
      if (l) l[i] = __float2bfloat16_rn(f - __bfloat162float(hb));
    }
  }
}

template <typename T>
int launch_cg_init(const T *B, T *X, T *R, T *P, int64_t ld, int64_t n, int64_t p,
                   __nv_bfloat16 *hi, __nv_bfloat16 *lo, double *partials, unsigned *counters,
                   double tol2, double atol2, double *rs, double *thr, int *iters, cudaStream_t s) {
  if (p <= 0 || n <= 0) return MFG_OK;
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  const int64_t nch = num_chunks<T>(n);
  cg_init_kernel<T><<<dim3((unsigned)nch, (unsigned)p), kThreads, 0, s>>>(
      B, X, R, P, ld, n, hi, lo, (int)nch, partials, counters, tol2, atol2, rs, thr, iters);
  return MFG_LAUNCH_STATUS();
}

template <typename T>
int launch_cg_update(T *X, T *R, const T *P, const T *W, int64_t ld, int64_t n, int64_t p,
                     const double *rs, const double *pap, const double *thr, double *partials,
                     unsigned *counters, double *rs_next, int *nactive, int *nactive_clear,
                     int *iters, cudaStream_t s) {
  if (p <= 0 || n <= 0) return MFG_OK;
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  const int64_t nch = num_chunks<T>(n);
  cg_update_kernel<T><<<dim3((unsigned)nch, (unsigned)p), kThreads, 0, s>>>(
      X, R, P, W, ld, n, rs, pap, thr, (int)nch, partials, counters, rs_next, nactive,
      nactive_clear, iters);
  return MFG_LAUNCH_STATUS();
}

template <typename T>
int launch_cg_step_small(T *X, T *R, T *P, const T *W, int64_t ld, int64_t n, int64_t p,
                         const double *rs, const double *thr, double *rs_next, int *nactive,
                         int *nactive_clear, int *iters, __nv_bfloat16 *hi, __nv_bfloat16 *lo,
                         cudaStream_t s) {
  if (p <= 0 || n <= 0) return MFG_OK;
  if (n > kCgSmallMaxN || p > 0x7fffffff) return MFG_ERR_UNSUPPORTED;
  static_assert(kCgSmallMaxN == 8 * kCgSmallThreads, "elements per thread");
  const unsigned grid = (unsigned)p;
  if (n <= kCgSmallThreads)
    cg_step_small_kernel<T, 1><<<grid, kCgSmallThreads, 0, s>>>(
        X, R, P, W, ld, n, rs, thr, rs_next, nactive, nactive_clear, iters, hi, lo);
  else if (n <= 2 * kCgSmallThreads)
    cg_step_small_kernel<T, 2><<<grid, kCgSmallThreads, 0, s>>>(
        X, R, P, W, ld, n, rs, thr, rs_next, nactive, nactive_clear, iters, hi, lo);
  else if (n <= 4 * kCgSmallThreads)
    cg_step_small_kernel<T, 4><<<grid, kCgSmallThreads, 0, s>>>(
        X, R, P, W, ld, n, rs, thr, rs_next, nactive, nactive_clear, iters, hi, lo);
  else
    cg_step_small_kernel<T, 8><<<grid, kCgSmallThreads, 0, s>>>(
        X, R, P, W, ld, n, rs, thr, rs_next, nactive, nactive_clear, iters, hi, lo);
  return MFG_LAUNCH_STATUS();
}

template <typename T>
int launch_cg_direction(T *P, const T *R, int64_t ld, int64_t n, int64_t p, const double *rs,
                        const double *rs_next, const double *thr, __nv_bfloat16 *hi,
                        __nv_bfloat16 *lo, cudaStream_t s) {
  if (p <= 0 || n <= 0) return MFG_OK;
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  const int64_t nch = num_chunks<T>(n);
  cg_direction_kernel<T><<<dim3((unsigned)nch, (unsigned)p), kThreads, 0, s>>>(
      P, R, ld, n, rs, rs_next, thr, hi, lo);
  return MFG_LAUNCH_STATUS();
}

// ---------------------------------------------------------------------------
// Two-sweep Arnoldi step (reortho = full, float bases of up to 64 vectors).
//
// The reference's step j (decomp.py:454-477) reads the basis three times:
// h = Q^T w, w' = w - Q h, w'' = w' - Q (Q^T w'), ||w''||.  Here the second
// projection of step j-1 is done in step j, over the same two reads of the
// basis as step j's own first projection.  The operator is applied to
// qt_j = u_j / nu_j, u_j = w'_{j-1} (first-projected, not yet
// reorthogonalised), and A q_j follows from the Arnoldi relation
// A Q_{j-1} = Q_j Hh (Hh: the full coefficients h + h2 and beta):
//   q_j = (u_j - Q h2) / beta,   A q_j = (nu_j A qt_j - Q_j Hh h2) / beta,
//   h_j = Q_j^T A q_j = (nu_j [g; q_j . A qt_j] - Hh h2) / beta,
//   w'_j = (I - Q_j Q_j^T) A q_j = (nu_j / beta) (I - Q_j Q_j^T) A qt_j.
// In exact arithmetic H, beta and the basis equal the reference's.  The
// rounding of A q_j grows with nu_j / beta_{j-1}, i.e. with the size of the
// second projection; when ||Q^T qt_j|| exceeds 0.1 (a vector that one
// projection left largely inside the basis, near an invariant subspace) the
// step raises MFG_ERR_RETRY and the caller repeats the solve with the
// three-sweep form.
// ---------------------------------------------------------------------------

// Basis vectors coff .. coff + ncols - 1 against a = w (per probe rows of
// w_bstride) and b = qt: out[b] = [Q^T qt (ncols) | at koff: Q^T w (ncols) | at
// 2 koff: qt . w], the last into cross[b * cross_bstride] instead when cross
// is given.
template <typename T>
int launch_proj2(const T *Q, int64_t q_bstride, int64_t q_istride, int coff, int ncols,
                 const T *Wa, const T *Wb, int64_t w_bstride, int64_t n, int64_t p,
                 double *partials, unsigned *counters, double *out, int64_t out_bstride,
                 int64_t koff, double *cross, int64_t cross_bstride, int *status, cudaStream_t s) {
  if (ncols <= 0 || p <= 0) return MFG_OK;
  StreamArgs a{Q,        q_bstride,   q_istride, ncols,   nullptr,  0,       0,
               const_cast<T *>(Wa), w_bstride, n,       p,        partials, counters,
               out,      out_bstride, 1,         cross,   cross_bstride, status};
  a.Wv2 = Wb;
  a.w2_bstride = w_bstride;
  a.koff = koff;
  a.coff = coff;
  return launch_stream_sweep<T, kStreamProj2>(a, s);
}

// Basis vectors coff .. coff + ncols - 1: Wa <- Wa - Q g (coef + koff),
// Wo <- Wb - Q h (coef); dots[b] = (||Wo||^2, ||Wa||^2, Wo . Wa).  Wo may be Wb.
template <typename T>
int launch_sub2(const T *Q, int64_t q_bstride, int64_t q_istride, int coff, int ncols,
                const double *coef, int64_t c_bstride, int64_t koff, T *Wa, int64_t wa_bstride,
                const T *Wb, int64_t wb_bstride, T *Wo, int64_t wo_bstride, int64_t n, int64_t p,
                double *partials, unsigned *counters, double *dots, int *status, cudaStream_t s) {
  if (ncols <= 0 || p <= 0) return MFG_OK;
  StreamArgs a{Q,  q_bstride,  q_istride, ncols,   coef,     c_bstride, 1,
               Wa, wa_bstride, n,         p,       partials, counters,  dots,
               3,  1,          nullptr,   0,       status};
  a.Wv2 = Wb;
  a.w2_bstride = wb_bstride;
  a.Wo2 = Wo;
  a.wo2_bstride = wo_bstride;
  a.koff = koff;
  a.coff = coff;
  return launch_stream_sweep<T, kStreamSub2>(a, s);
}

// One CTA of four warps per probe: the coefficient algebra of step j >= 1
// (see above).
// X2: [Q^T qt (j) | Q^T w (j) at koff | qt . w at 2 koff], dots: (||b'||^2,
// ||z||^2, b' . z) with b' = qt - Q Q^T qt, z = w - Q Q^T w.  Writes H row/col
// entries of the reference's H, the full coefficients Hh ((k + 1) x k), the
// next scale nu and the finish coefficients cf = (1/rho, 1/s, qw/(rho s)).
// Hh is stored column-major ((k + 1) rows a column) so that a column update
// and the product Hh h2 read and write consecutive words across the lanes.
// The product's stored columns 0 .. j - 2 are cut into four contiguous
// ranges, one per warp (a quarter of the dependent load rounds); warp 0 adds
// the four partial sums in warp order and finishes alone.
constexpr int kCoefWarps = 4;

__global__ void __launch_bounds__(32 * kCoefWarps)
twosweep_coef_kernel(int j, int k, int64_t p, const double *__restrict__ X2, int64_t koff,
                     const double *__restrict__ dots, double *__restrict__ H,
                     double *__restrict__ Hh, double *__restrict__ nu, double *__restrict__ cf,
                     int *__restrict__ status) {
  // j <= kTwoSweepMaxK - 1 = 128: columns in 4 blocks of 32 lanes, rows
  // (0 .. j) in 5 blocks
  constexpr int kCB = 4, kRB = 5;
  __shared__ double msum[kCoefWarps][kRB * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t b = blockIdx.x;
  if (b >= p) return;  // block-uniform
  const double *x = X2 + b * (2 * koff + 1);
  double *Hb = H + b * (int64_t)k * k;
  double *Hhb = Hh + b * (int64_t)(k + 1) * k;  // column-major: column l at Hhb + l (k + 1)
  const int64_t ld = k + 1;
  // warp 0: every input of the finishing algebra first, in one round of
  // independent loads; all warps: Q^T qt (the product's vector)
  double nb = 0.0, nz = 0.0, bz = 0.0, c = 0.0, nuj = 0.0;
  double hq[kCB], g[kCB], hp[kCB];
  if (warp == 0) {
    nb = dots[b * 3];
    nz = dots[b * 3 + 1];
    bz = dots[b * 3 + 2];
    c = x[2 * koff];
    nuj = nu[b];
  }
#pragma unroll
  for (int cb = 0; cb < kCB; ++cb) {
    const int l = lane + 32 * cb;
    const bool ok = l < j;
    hq[cb] = ok ? x[l] : 0.0;
    g[cb] = (ok && warp == 0) ? x[koff + l] : 0.0;
    hp[cb] = (ok && warp == 0) ? Hb[(int64_t)l * k + (j - 1)] : 0.0;
  }
  if (j < k) {
    // partial m = Hh[0:j+1, cols] hq over this warp's columns: all lanes walk
    // the same columns (hq_l broadcast by shuffle), eight columns of loads
    // in flight; entries below the subdiagonal (never written) are masked
    const int ncol = j - 1;
    const int per = (ncol + kCoefWarps - 1) / kCoefWarps;
    const int lb = warp * per;
    const int le = lb + per < ncol ? lb + per : ncol;
    double m[kRB];
#pragma unroll
    for (int r = 0; r < kRB; ++r) m[r] = 0.0;
    for (int l0 = lb; l0 < le; l0 += 8) {
      double a[8][kRB];
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int l = l0 + t;
        const double *cl = Hhb + (int64_t)l * ld;
#pragma unroll
        for (int r = 0; r < kRB; ++r) {
          const int i = lane + 32 * r;
          a[t][r] = (l < le && i <= l + 1) ? cl[i] : 0.0;
        }
      }
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        const int l = l0 + t;
        const double src = l < 32 ? hq[0] : (l < 64 ? hq[1] : (l < 96 ? hq[2] : hq[3]));
        const double hv = __shfl_sync(0xffffffffu, src, l & 31);
#pragma unroll
        for (int r = 0; r < kRB; ++r) m[r] = fma(a[t][r], hv, m[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < kRB; ++r) msum[warp][r * 32 + lane] = m[r];
  }
  __syncthreads();
  if (warp != 0) return;
  double hh = 0.0, hg = 0.0;
#pragma unroll
  for (int cb = 0; cb < kCB; ++cb) {
    hh = fma(hq[cb], hq[cb], hh);
    hg = fma(hq[cb], g[cb], hg);
  }
  hh = warp_sum(hh);
  hg = warp_sum(hg);
  const double rho = sqrt(nb);   // ||w''_{j-1}|| / nu_j
  const double beta = nuj * rho;
  // column j-1 of Hh (the reference's h_{j-1} plus the second projection,
  // beta below it) for the rows lane + 32 r, kept in registers
  double cj[kRB];
#pragma unroll
  for (int r = 0; r < kRB; ++r) {
    const int i = lane + 32 * r;
    const double up = r < kCB ? hp[r < kCB ? r : 0] + nuj * hq[r < kCB ? r : 0] : 0.0;
    cj[r] = i < j ? up : (i == j ? beta : 0.0);
  }
  double *col = Hhb + (int64_t)(j - 1) * ld;
#pragma unroll
  for (int r = 0; r < kRB; ++r)
    if (lane + 32 * r <= j) col[lane + 32 * r] = cj[r];
  if (lane == 0) Hb[(int64_t)j * k + (j - 1)] = beta;
  const double qw = (c - hg) / rho;  // q_j . A qt_j
  if (j < k) {
    double m[kRB];
#pragma unroll
    for (int r = 0; r < kRB; ++r) {
      m[r] = msum[0][r * 32 + lane];
#pragma unroll
      for (int w = 1; w < kCoefWarps; ++w) m[r] += msum[w][r * 32 + lane];
    }
    {
      const int l = j - 1;
      const double src = l < 32 ? hq[0] : (l < 64 ? hq[1] : (l < 96 ? hq[2] : hq[3]));
      const double hv = __shfl_sync(0xffffffffu, src, l & 31);
#pragma unroll
      for (int r = 0; r < kRB; ++r) m[r] = fma(cj[r], hv, m[r]);
    }
    // h_j = (nu [g; qw] - m) / beta into column j of H
#pragma unroll
    for (int r = 0; r < kRB; ++r) {
      const int i = lane + 32 * r;
      if (i <= j) {
        const double top = (r < kCB && i < j) ? g[r < kCB ? r : 0] : qw;
        Hb[(int64_t)i * k + j] = nuj * (top - m[r]) / beta;
      }
    }
  }
  if (lane == 0) {
    if (hh > 0.01 * (hh + nb) && status) atomicExch(status, (int)MFG_ERR_RETRY);
    // y = z - q_j qw, ||y||^2 = ||z||^2 - 2 qw (q_j . z) + qw^2
    const double qz = bz / rho;
    const double s2 = nz - 2.0 * qw * qz + qw * qw;
    const double sy = s2 > 1e-12 * nz ? sqrt(s2) : sqrt(nz);
    nu[b] = sy / rho;  // u_{j+1} = y / rho = nu_{j+1} qt_{j+1}
    cf[b * 4] = 1.0 / rho;
    cf[b * 4 + 1] = 1.0 / sy;
    cf[b * 4 + 2] = qw / (rho * sy);
  }
}

// End of step j: q_j = b' / rho in place; qt_{j+1} = z / s - b' qw / (rho s)
// (float copy and bf16 hi/lo) unless qt is null.
template <typename T>
__global__ void __launch_bounds__(kThreads)
twosweep_finish_kernel(T *__restrict__ Qj, int64_t q_bstride, const T *__restrict__ Z,
                       int64_t w_bstride, int64_t n, const double *__restrict__ cf,
                       T *__restrict__ qt, __nv_bfloat16 *__restrict__ hi,
                       __nv_bfloat16 *__restrict__ lo, int64_t bf_bstride) {
  constexpr int W = Vec<T>::width;
  const int64_t c = blockIdx.x;
  const int64_t b = blockIdx.y;
  const T t1 = (T)cf[b * 4], cz = (T)cf[b * 4 + 1], cb = (T)cf[b * 4 + 2];
  T bv[kVPT][W], zv[kVPT][W];
  load_chunk<T>(Qj + b * q_bstride, n, c, bv);
  if (qt) load_chunk<T>(Z + b * w_bstride, n, c, zv);
#pragma unroll
  for (int e = 0; e < kVPT; ++e)
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const T bb = bv[e][u];
      bv[e][u] = bb * t1;
      if (qt) zv[e][u] = zv[e][u] * cz - bb * cb;
    }
  store_chunk<T>(Qj + b * q_bstride, n, c, bv);
  if (!qt) return;
  store_chunk<T>(qt + b * w_bstride, n, c, zv);
  if (hi == nullptr) return;
#pragma unroll
  for (int e = 0; e < kVPT; ++e) {
    const int64_t r = c * chunk_rows<T>() + ((int64_t)e * kThreads + threadIdx.x) * W;
    if (r >= n) continue;
    __nv_bfloat16 h[W], l[W];
#pragma unroll
    for (int u = 0; u < W; ++u) {
      const float xv = (float)zv[e][u];
      h[u] = __float2bfloat16_rn(xv);
      l[u] = __float2bfloat16_rn(xv - __bfloat162float(h[u]));
    }
    if constexpr (W == 4) {
      uint2 hv, lv;
      hv.x = (uint32_t)__bfloat16_as_ushort(h[0]) | ((uint32_t)__bfloat16_as_ushort(h[1]) << 16);
      hv.y = (uint32_t)__bfloat16_as_ushort(h[2]) | ((uint32_t)__bfloat16_as_ushort(h[3]) << 16);
      lv.x = (uint32_t)__bfloat16_as_ushort(l[0]) | ((uint32_t)__bfloat16_as_ushort(l[1]) << 16);
      lv.y = (uint32_t)__bfloat16_as_ushort(l[2]) | ((uint32_t)__bfloat16_as_ushort(l[3]) << 16);
      *reinterpret_cast<uint2 *>(hi + b * bf_bstride + r) = hv;
      if (lo) *reinterpret_cast<uint2 *>(lo + b * bf_bstride + r) = lv;
    } else {
#pragma unroll
      for (int u = 0; u < W; ++u) {
        hi[b * bf_bstride + r + u] = h[u];
        if (lo) lo[b * bf_bstride + r + u] = l[u];
      }
    }
  }
}

int launch_twosweep_coef(int j, int k, int64_t p, const double *X2, int64_t koff,
                         const double *dots, double *H, double *Hh, double *nu, double *cf,
                         int *status, cudaStream_t s) {
  if (p <= 0) return MFG_OK;
  if (p > 2147483647) return MFG_ERR_UNSUPPORTED;
  twosweep_coef_kernel<<<(unsigned)p, 32 * kCoefWarps, 0, s>>>(j, k, p, X2, koff, dots, H, Hh, nu,
                                                               cf, status);
  return MFG_LAUNCH_STATUS();
}

template <typename T>
int launch_twosweep_finish(T *Qj, int64_t q_bstride, const T *Z, int64_t w_bstride, int64_t n,
                           int64_t p, const double *cf, T *qt, __nv_bfloat16 *hi,
                           __nv_bfloat16 *lo, int64_t bf_bstride, cudaStream_t s) {
  if (p <= 0) return MFG_OK;
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)num_chunks<T>(n), (unsigned)p);
  twosweep_finish_kernel<T><<<grid, kThreads, 0, s>>>(Qj, q_bstride, Z, w_bstride, n, cf, qt, hi,
                                                      lo, bf_bstride);
  return MFG_LAUNCH_STATUS();
}

template int launch_proj2<float>(const float *, int64_t, int64_t, int, int, const float *,
                                 const float *, int64_t, int64_t, int64_t, double *, unsigned *,
                                 double *, int64_t, int64_t, double *, int64_t, int *,
                                 cudaStream_t);
template int launch_sub2<float>(const float *, int64_t, int64_t, int, int, const double *,
                                int64_t, int64_t, float *, int64_t, const float *, int64_t,
                                float *, int64_t, int64_t, int64_t, double *, unsigned *,
                                double *, int *, cudaStream_t);
template int launch_twosweep_finish<float>(float *, int64_t, const float *, int64_t, int64_t,
                                           int64_t, const double *, float *, __nv_bfloat16 *,
                                           __nv_bfloat16 *, int64_t, cudaStream_t);

#define MFG_INST(T)                                                                          \
  template int launch_cg_init<T>(const T *, T *, T *, T *, int64_t, int64_t, int64_t,         \
                                 __nv_bfloat16 *, __nv_bfloat16 *, double *, unsigned *,      \
                                 double, double, double *, double *, int *, cudaStream_t);    \
  template int launch_cg_update<T>(T *, T *, const T *, const T *, int64_t, int64_t, int64_t,  \
                                   const double *, const double *, const double *, double *,  \
                                   unsigned *, double *, int *, int *, int *, cudaStream_t);  \
  template int launch_cg_step_small<T>(T *, T *, T *, const T *, int64_t, int64_t, int64_t,     \
                                       const double *, const double *, double *, int *, int *, \
                                       int *, __nv_bfloat16 *, __nv_bfloat16 *, cudaStream_t); \
  template int launch_cg_direction<T>(T *, const T *, int64_t, int64_t, int64_t,              \
                                      const double *, const double *, const double *,         \
                                      __nv_bfloat16 *, __nv_bfloat16 *, cudaStream_t);        \
  template int sub_proj_rows_per_thread<T>(int);                                               \
  template int64_t max_fused_chunks<T>(int64_t);                                               \
  template int launch_sub_proj<T>(const T *, int64_t, int64_t, int, const double *, int64_t,   \
                                  int64_t, T *, int64_t, int64_t, int64_t, double *,           \
                                  unsigned *, double *, int64_t, int *, cudaStream_t);         \
  template int launch_proj<T>(const T *, int64_t, int64_t, int, const T *, int64_t, int64_t,   \
                              int64_t, double *, unsigned *, double *, int64_t, int64_t,       \
                              cudaStream_t, int *);                                            \
  template int launch_sub<T>(const T *, int64_t, int64_t, int, const double *, int64_t,        \
                             int64_t, const T *, T *, int64_t, int64_t, int64_t, bool, bool,   \
                             double *, unsigned *, double *, double *, int64_t, cudaStream_t,  \
                             int *);                                                           \
  template int launch_scale<T>(const T *, int64_t, int64_t, int64_t, const double *, T *,      \
                               int64_t, __nv_bfloat16 *, __nv_bfloat16 *, int64_t, cudaStream_t);
MFG_INST(float)
MFG_INST(double)
#undef MFG_INST

}  // namespace mfg
