// Shared helpers of the matfree_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/matfree_gb300.h"

namespace mfg {
// Records the call site and CUDA error text of the most recent failure on
// this host thread (read back through mfg_last_error()).
void record_error(const char *where, int line, const char *what);
inline int cuda_status(cudaError_t e, const char *where, int line) {
  if (e == cudaSuccess) return MFG_OK;
  record_error(where, line, cudaGetErrorString(e));
  return MFG_ERR_CUDA;
}
}  // namespace mfg

#define MFG_CUDA_TRY(expr)                                                  \
  do {                                                                      \
    const int _s = ::mfg::cuda_status((expr), __FILE__, __LINE__);          \
    if (_s != MFG_OK) return _s;                                            \
  } while (0)

// status of the kernel launch just issued (configuration errors, and sticky
// errors of earlier kernels on the device)
#define MFG_LAUNCH_STATUS() ::mfg::cuda_status(cudaGetLastError(), __FILE__, __LINE__)

#define MFG_TRY(expr)                                       \
  do {                                                      \
    int _s = (expr);                                        \
    if (_s != MFG_OK) return _s;                            \
  } while (0)

namespace mfg {

constexpr int kThreads = 256;  // threads per CTA of the streaming kernels
constexpr int kWarps = kThreads / 32;

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------
// mbarrier waits, bounded in wall-clock time (%globaltimer) and given up
// early when another role raised the CTA's failure flag.  Waits on the
// critical path poll mbarrier.try_wait; waits of idle roles (an epilogue
// waiting for the whole main loop) sleep in it with a suspend-time hint, so
// they take no issue slots from the warps doing the work.
// ---------------------------------------------------------------------------

constexpr uint64_t kMbarWaitNs = 2000000000ull;  // 2 s: far beyond any copy or MMA
constexpr uint32_t kMbarSleepNs = 1000000u;      // per sleeping try_wait

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <bool kSleep>
__device__ __forceinline__ bool mbar_try_wait_parity(uint32_t bar_saddr, uint32_t parity) {
  uint32_t ok;
  if constexpr (kSleep) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar_saddr), "r"(parity), "r"(kMbarSleepNs)
        : "memory");
  } else {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar_saddr), "r"(parity)
        : "memory");
  }
  return ok != 0;
}

// True once the phase of the barrier at shared address `bar_saddr` with the
// given parity has completed; false after `limit_ns` or when *fail (if given)
// becomes non-zero.
template <bool kSleep = false>
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar_saddr, uint32_t parity,
                                                  volatile int *fail,
                                                  uint64_t limit_ns = kMbarWaitNs) {
  if (mbar_try_wait_parity<kSleep>(bar_saddr, parity)) return true;
  const uint64_t t0 = global_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait_parity<kSleep>(bar_saddr, parity)) return true;
    if (kSleep || (it & 63u) == 0) {
      if (fail && *fail) return false;
      if (global_ns() - t0 > limit_ns) return false;
    }
  }
}
inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// 16-byte vector type per element type: 4 floats or 2 doubles.
template <typename T> struct Vec;
template <> struct Vec<float> {
  using type = float4;
  static constexpr int width = 4;
};
template <> struct Vec<double> {
  using type = double2;
  static constexpr int width = 2;
};

template <typename T>
__device__ __forceinline__ void vec_to_array(const typename Vec<T>::type &v, T *a);
template <>
__device__ __forceinline__ void vec_to_array<float>(const float4 &v, float *a) {
  a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w;
}
template <>
__device__ __forceinline__ void vec_to_array<double>(const double2 &v, double *a) {
  a[0] = v.x; a[1] = v.y;
}
template <typename T>
__device__ __forceinline__ typename Vec<T>::type array_to_vec(const T *a);
template <>
__device__ __forceinline__ float4 array_to_vec<float>(const float *a) {
  return make_float4(a[0], a[1], a[2], a[3]);
}
template <>
__device__ __forceinline__ double2 array_to_vec<double>(const double *a) {
  return make_double2(a[0], a[1]);
}

// Accumulator type of the per-thread partial sums: float32 for float data
// (combined in float64 across threads), float64 for double data.
template <typename T> struct Acc { using type = T; };

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace mfg
