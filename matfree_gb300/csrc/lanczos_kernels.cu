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

// ---------------------------------------------------------------------------
// Fused second pass: w' = w - Q c, then h2 = Q^T w' from one read of Q.
//
// The CTA owns R = kThreads * EPT consecutive rows of one probe.  One thread
// issues a bulk asynchronous copy per basis vector (its R-row segment) into
// shared memory, all completing on one mbarrier; the CTA then forms w' from
// shared memory, stores it, and reads the same shared tile again for the
// projections.  This removes one of the four basis sweeps of a CGS2 step.
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

constexpr uint32_t kBarWaitLimit = 1u << 24;
constexpr int kSPGroup = 8;                                    // columns per copy barrier
constexpr int kMaxSPGroups = (kMaxProjCols + kSPGroup - 1) / kSPGroup;
constexpr size_t kSubProjSmemBudget = 110 * 1024;              // two CTAs per SM

__device__ __forceinline__ bool bar_try_wait0(uint64_t *bar) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar))
      : "memory");
  return ok != 0;
}

// Basis tile loads: full groups of kSPGroup vectors arrive as one 2-D tensor
// copy (box of R rows x kSPGroup vectors, rows past n zero-filled); a tail of
// fewer than kSPGroup vectors arrives as one 1-D bulk copy per vector.
template <typename T, int EPT>
__global__ void __launch_bounds__(kThreads)
sub_proj_kernel(const __grid_constant__ CUtensorMap qmap, const T *__restrict__ Q,
                int64_t q_bstride, int64_t q_istride, int ncols,
                const double *__restrict__ coef, int64_t c_bstride, int64_t c_istride,
                T *Wv, int64_t w_bstride, int64_t n, int nchunks, double *__restrict__ partials,
                unsigned *__restrict__ counters, double *__restrict__ out, int64_t out_bstride,
                int *__restrict__ status) {
  constexpr int R = kThreads * EPT;
  extern __shared__ __align__(128) uint8_t smem[];
  T *qs = reinterpret_cast<T *>(smem);                       // [ncols][R]
  T *ws = qs + (size_t)ncols * R;                            // [R]  w' of this chunk
  T *s_coef = ws + R;                                        // [ncols]
  double *red = reinterpret_cast<double *>(s_coef + ((ncols + 1) & ~1));  // [ncols]
  __shared__ __align__(8) uint64_t bars[kMaxSPGroups];
  __shared__ int s_fail;

  const int64_t c = blockIdx.x;
  const int64_t b = blockIdx.y;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t r0 = c * R;
  const int64_t rows = (n - r0 < R) ? (n - r0) : R;
  const uint32_t seg_bytes = (uint32_t)(((rows * (int64_t)sizeof(T)) + 15) / 16 * 16);
  const int ngroups = (ncols + kSPGroup - 1) / kSPGroup;

  if (threadIdx.x == 0) {
    for (int g = 0; g < ngroups; ++g)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&bars[g])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    s_fail = 0;
  }
  __syncthreads();
  if (warp == 0) {
    // one barrier per group of columns: the update consumes columns as they
    // land.  Lane 0 arms every barrier and issues the 2-D tile copies of the
    // full groups; the lanes issue the 1-D copies of the tail vectors.
    // 2-D tensor copies need a 128-byte aligned shared destination; if the
    // tile is not aligned, record it and load every vector with 1-D copies.
    const bool tile_ok = (smem_addr(qs) & 127u) == 0;
    if (!tile_ok && lane == 0 && status) atomicExch(status, (int)MFG_ERR_BAD_ARG);
    const int full = tile_ok ? ncols / kSPGroup : 0;
    const int kcols = (int)(q_bstride / q_istride);  // basis vectors per probe
    if (lane == 0) {
      for (int g = 0; g < ngroups; ++g) {
        const bool is_full = g < full;
        const uint32_t bytes = is_full ? (uint32_t)(kSPGroup * R * sizeof(T))
                                       : seg_bytes * (uint32_t)(ncols - g * kSPGroup);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                         smem_addr(&bars[g])),
                     "r"(bytes)
                     : "memory");
        if (is_full) {
          const int x = (int)r0, y = (int)(b * kcols + g * kSPGroup);
          asm volatile(
              "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
              "[%0], [%1, {%3, %4}], [%2];" ::"r"(smem_addr(qs + (size_t)g * kSPGroup * R)),
              "l"(reinterpret_cast<uint64_t>(&qmap)), "r"(smem_addr(&bars[g])), "r"(x), "r"(y)
              : "memory");
        }
      }
    }
    __syncwarp();
    for (int i = full * kSPGroup + lane; i < ncols; i += 32) {
      const T *src = Q + b * q_bstride + (int64_t)i * q_istride + r0;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
          ::"r"(smem_addr(qs + (size_t)i * R)), "l"(reinterpret_cast<uint64_t>(src)),
          "r"(seg_bytes), "r"(smem_addr(&bars[i / kSPGroup]))
          : "memory");
    }
  }
  for (int i = threadIdx.x; i < ncols; i += kThreads) s_coef[i] = (T)coef[b * c_bstride + i * c_istride];

  // this thread's EPT consecutive rows
  const int64_t rt = r0 + (int64_t)threadIdx.x * EPT;
  T w[EPT];
#pragma unroll
  for (int e = 0; e < EPT; ++e) w[e] = (rt + e < n) ? Wv[b * w_bstride + rt + e] : (T)0;
  __syncthreads();

  const T *qrow = qs + (size_t)threadIdx.x * EPT;
  volatile int *fail = &s_fail;
  for (int g = 0; g < ngroups; ++g) {
    // bounded wait for this group's basis segments
    bool ready = false;
    for (uint32_t it = 0; it < kBarWaitLimit; ++it) {
      if (bar_try_wait0(&bars[g])) {
        ready = true;
        break;
      }
      if ((it & 1023u) == 1023u && *fail) break;
    }
    if (!ready) {
      *fail = 1;
      if (status) atomicExch(status, (int)MFG_ERR_TIMEOUT);
      break;
    }
    const int i1 = (g + 1) * kSPGroup < ncols ? (g + 1) * kSPGroup : ncols;
    for (int i = g * kSPGroup; i < i1; ++i) {
      const T ci = s_coef[i];
#pragma unroll
      for (int e = 0; e < EPT; ++e) w[e] = fma(-qrow[(size_t)i * R + e], ci, w[e]);
    }
  }
  __syncthreads();
  if (s_fail) return;
#pragma unroll
  for (int e = 0; e < EPT; ++e) {
    if (rt + e < n) Wv[b * w_bstride + rt + e] = w[e];
    ws[threadIdx.x * EPT + e] = (rt + e < n) ? w[e] : (T)0;
  }
  __syncthreads();

  // h2: warp `warp` owns columns warp, warp + 8, ...; its lanes stride the
  // R rows of the chunk, so one warp reduction covers R products.  Rows past
  // n hold stale shared memory and are left out.
  for (int i = warp; i < ncols; i += kWarps) {
    const T *col = qs + (size_t)i * R;
    T acc = (T)0;
#pragma unroll 4
    for (int r = lane; r < R; r += 32)
      if (r < rows) acc = fma(col[r], ws[r], acc);
    acc = warp_sum_t<T>(acc);
    if (lane == 0) red[i] = (double)acc;
  }
  __syncthreads();
  finish_columns(red, ncols, b, c, nchunks, partials, counters, out, out_bstride, 1, 1);
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
  if (p > 65535 || ncols > kMaxProjCols) return MFG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)nch, (unsigned)p);
  const size_t smem = (size_t)ncols * kWarps * sizeof(double);
  proj_kernel<T><<<grid, kThreads, smem, s>>>(Q, q_bstride, q_istride, ncols, Wv, w_bstride, n,
                                              (int)nch, partials, counters, out, out_bstride,
                                              out_istride);
  return MFG_LAUNCH_STATUS();
}

// Rows per CTA of the fused kernel: the largest of 4/2/1 rows per thread
// (width-limited for doubles) whose basis tile fits the shared-memory budget.
// shared memory of the fused kernel: basis tile, w' tile, coefficients, column sums
template <typename T>
static size_t sub_proj_smem(int ncols, int64_t R) {
  return (size_t)ncols * R * sizeof(T) + (size_t)R * sizeof(T) + (size_t)(ncols + 2) * sizeof(T) +
         (size_t)ncols * sizeof(double);
}

// One row per thread: the 2-D tile copies load R = 256 rows per vector.
template <typename T>
int sub_proj_rows_per_thread(int ncols) {
  if (ncols > kMaxProjCols) return 0;
  return sub_proj_smem<T>(ncols, (int64_t)kThreads) <= kSubProjSmemBudget ? 1 : 0;
}

template <typename T> int64_t max_fused_chunks(int64_t n) { return ceil_div(n, kThreads); }

template <typename T, int EPT>
static int launch_sub_proj_t(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols,
                             const double *coef, int64_t c_bstride, int64_t c_istride, T *Wv,
                             int64_t w_bstride, int64_t n, int64_t p, double *partials,
                             unsigned *counters, double *out, int64_t out_bstride, int *status,
                             cudaStream_t s) {
  const int64_t R = (int64_t)kThreads * EPT;
  const int64_t nch = ceil_div(n, R);
  const size_t smem = sub_proj_smem<T>(ncols, R);
  if (q_istride <= 0 || q_bstride % q_istride != 0) return MFG_ERR_BAD_ARG;
  // the basis as rows of q_istride elements: row b * k + i is probe b's vector i
  CUtensorMap qmap;
  const int64_t kcols = q_bstride / q_istride;
  if (!make_plain_tensor_map_2d(&qmap, (int)sizeof(T), Q, n, p * kcols, q_istride, (uint32_t)R,
                                (uint32_t)kSPGroup))
    return MFG_ERR_CUDA;
  const cudaError_t before = cudaGetLastError();
  // The default dynamic limit is 48 KB minus the kernel's static shared
  // memory, so the opt-in is raised well below 48 KB.
  if (smem > 32 * 1024)
    MFG_CUDA_TRY(cudaFuncSetAttribute(sub_proj_kernel<T, EPT>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 grid((unsigned)nch, (unsigned)p);
  sub_proj_kernel<T, EPT><<<grid, kThreads, smem, s>>>(qmap, Q, q_bstride, q_istride, ncols, coef,
                                                       c_bstride, c_istride, Wv, w_bstride, n,
                                                       (int)nch, partials, counters, out,
                                                       out_bstride, status);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFuncAttributes fa{};
    cudaFuncGetAttributes(&fa, sub_proj_kernel<T, EPT>);
    char msg[256];
    snprintf(msg, sizeof(msg), "%s (smem %zu, maxDyn %d, static %zu, grid %ux%u, ncols %d, before %s)",
             cudaGetErrorString(e), smem, fa.maxDynamicSharedSizeBytes, fa.sharedSizeBytes, grid.x,
             grid.y, ncols, cudaGetErrorString(before));
    record_error(__FILE__, __LINE__, msg);
    return MFG_ERR_CUDA;
  }
  return MFG_OK;
}

template <typename T>
int launch_sub_proj(const T *Q, int64_t q_bstride, int64_t q_istride, int ncols, const double *coef,
                    int64_t c_bstride, int64_t c_istride, T *Wv, int64_t w_bstride, int64_t n,
                    int64_t p, double *partials, unsigned *counters, double *out,
                    int64_t out_bstride, int *status, cudaStream_t s) {
  if (ncols <= 0 || p <= 0) return MFG_OK;
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  const int ept = sub_proj_rows_per_thread<T>(ncols);
  if (ept == 1)
    return launch_sub_proj_t<T, 1>(Q, q_bstride, q_istride, ncols, coef, c_bstride, c_istride, Wv,
                                   w_bstride, n, p, partials, counters, out, out_bstride, status, s);
  return MFG_ERR_UNSUPPORTED;
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

#define MFG_INST(T)                                                                          \
  template int sub_proj_rows_per_thread<T>(int);                                               \
  template int64_t max_fused_chunks<T>(int64_t);                                               \
  template int launch_sub_proj<T>(const T *, int64_t, int64_t, int, const double *, int64_t,   \
                                  int64_t, T *, int64_t, int64_t, int64_t, double *,           \
                                  unsigned *, double *, int64_t, int *, cudaStream_t);         \
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
