// Self-test of the bounded device-side waits (failure detection without a
// GPU fault).
//
// Every spin in this library's kernels (TMA copy completions, MMA commits,
// copy-warp / consumer hand-offs) goes through mbar_wait_bounded: a wait
// that gives up after a wall-clock limit, or early when another role of the
// CTA raised the shared failure flag, after which the kernel records
// MFG_ERR_TIMEOUT in a device status word and returns.  This kernel runs that
// protocol on an mbarrier nothing ever arrives on, with no copy in flight
// and no tensor memory held, so the wait always runs out and nothing else
// can go wrong:
//   warp 0 (the "producer")  polls the barrier (the critical-path form) for
//                            `limit_ns`, then raises the failure flag and
//                            writes MFG_ERR_TIMEOUT to *status;
//   warp 1 (an idle role)    sleeps in try_wait (the form of epilogue
//                            warps) with the 2 s production limit, and must
//                            leave early through the failure flag.
// The host reads back the status and both warps' wait times.
#include "common.cuh"

namespace mfg {

__device__ __forceinline__ uint32_t selftest_smem(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__global__ void __launch_bounds__(64) wait_selftest_kernel(uint64_t limit_ns, int *status,
                                                           unsigned long long *out) {
  __shared__ __align__(8) uint64_t bar;
  __shared__ volatile int fail;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (threadIdx.x == 0) {
    fail = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(selftest_smem(&bar)), "r"(1u) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (lane == 0) {
    const uint64_t t0 = global_ns();
    bool ok;
    if (warp == 0) {
      ok = mbar_wait_bounded<false>(selftest_smem(&bar), 0u, &fail, limit_ns);
      if (!ok) {
        fail = 1;
        atomicExch(status, (int)MFG_ERR_TIMEOUT);
      }
    } else {
      ok = mbar_wait_bounded<true>(selftest_smem(&bar), 0u, &fail, kMbarWaitNs);
    }
    out[2 * warp] = (unsigned long long)(global_ns() - t0);
    out[2 * warp + 1] = ok ? 1ull : 0ull;
  }
  __syncthreads();
  if (threadIdx.x == 0) out[4] = (unsigned long long)fail;
}

int launch_wait_selftest(uint64_t limit_ns, int *status, unsigned long long *out, cudaStream_t s) {
  wait_selftest_kernel<<<1, 64, 0, s>>>(limit_ns, status, out);
  return MFG_LAUNCH_STATUS();
}

}  // namespace mfg
