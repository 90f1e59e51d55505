// Dense W = A V on the 5th-generation tensor cores (placeholder until the
// tcgen05 kernel lands; the bf16 precisions report MFG_ERR_UNSUPPORTED).
#include "common.cuh"
#include "kernels.cuh"

namespace mfg {

bool tcgen05_supported_shape(int64_t, int64_t) { return false; }

int launch_dense_tcgen05(const __nv_bfloat16 *, const __nv_bfloat16 *, int64_t,
                         const __nv_bfloat16 *, const __nv_bfloat16 *, int64_t, const float *,
                         int64_t, float *, int64_t, int64_t, int64_t, double, int *,
                         cudaStream_t) {
  return MFG_ERR_UNSUPPORTED;
}

}  // namespace mfg
