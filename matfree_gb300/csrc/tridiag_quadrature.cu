// Batched symmetric tridiagonal eigensolve + Gauss quadrature (float64).
//
// For each probe's k x k Hessenberg matrix H the kernel forms the symmetric
// tridiagonal T = (H + H^T)/2 (diagonal H_ii, off-diagonal (H_i,i+1 + H_i+1,i)/2),
// diagonalises it by the implicit QL method with Wilkinson shifts (Givens
// chase from the bottom of the unreduced block up to l), and tracks only the
// first row of the eigenvector matrix, as in the Golub-Welsch construction of
// Gauss rules.  The quadrature value is scale_b * sum_i f(lambda_i) s_1i^2,
// which equals e1^T V diag(f(lambda)) V^T e1 of the dense eigh route.
//
// One thread owns one problem; the three length-k work arrays live in shared
// memory with the thread index fastest, so the lanes of a warp touch
// consecutive words.  The sweep limit per eigenvalue is bounded; a problem
// that does not converge returns NaN and raises MFG_ERR_NO_CONVERGENCE.
#include <cfloat>

#include "common.cuh"
#include "kernels.cuh"

namespace mfg {

constexpr int kMaxSweeps = 64;

__global__ void tridiag_ql_kernel(int k, int64_t p, const double *__restrict__ H, int fun,
                                  double param, const double *__restrict__ scale,
                                  double *__restrict__ values, double *__restrict__ eigvals,
                                  double *__restrict__ first_sq, int *__restrict__ status) {
  extern __shared__ double sm[];
  const int TB = blockDim.x;
  const int t = threadIdx.x;
  const int64_t b = blockIdx.x * (int64_t)TB + t;
  if (b >= p) return;
  double *d = sm + t;
  double *e = sm + (size_t)TB * k + t;
  double *z = sm + (size_t)2 * TB * k + t;
#define D_(i) d[(size_t)(i) * TB]
#define E_(i) e[(size_t)(i) * TB]
#define Z_(i) z[(size_t)(i) * TB]
  const double *Hb = H + (size_t)b * k * k;
  for (int i = 0; i < k; ++i) {
    D_(i) = Hb[(size_t)i * k + i];
    E_(i) = (i + 1 < k) ? 0.5 * (Hb[(size_t)i * k + i + 1] + Hb[(size_t)(i + 1) * k + i]) : 0.0;
    Z_(i) = (i == 0) ? 1.0 : 0.0;
  }
  bool ok = true;
  for (int l = 0; l < k && ok; ++l) {
    int sweeps = 0;
    while (true) {
      int m = l;
      for (; m < k - 1; ++m) {
        const double dd = fabs(D_(m)) + fabs(D_(m + 1));
        if (fabs(E_(m)) <= DBL_EPSILON * dd) break;
      }
      if (m == l) break;
      if (++sweeps > kMaxSweeps) {
        ok = false;
        break;
      }
      // shift from the leading 2x2 block, in the numerically safe form
      double g = (D_(l + 1) - D_(l)) / (2.0 * E_(l));
      double r = hypot(g, 1.0);
      g = D_(m) - D_(l) + E_(l) / (g + copysign(r, g));
      double s = 1.0, c = 1.0, shift_acc = 0.0;
      bool deflated = false;
      // The chase reads d_i, e_i, z_i before they are written in this sweep,
      // and d_{i+1}, z_{i+1} as left by the previous rotation: those travel in
      // registers and the next rotation's inputs are loaded one step ahead, so
      // shared-memory latency stays off the float64 dependence chain.
      double d_up = D_(m), z_up = Z_(m);                // d_{i+1}, z_{i+1}
      double e_i = E_(m - 1), d_i = D_(m - 1), z_i = Z_(m - 1);
      for (int i = m - 1; i >= l; --i) {
        double e_nx = 0.0, d_nx = 0.0, z_nx = 0.0;
        if (i > l) {
          e_nx = E_(i - 1);
          d_nx = D_(i - 1);
          z_nx = Z_(i - 1);
        }
        const double f = s * e_i;
        const double bb = c * e_i;
        // Entries of Lanczos tridiagonals are far from the overflow range, so
        // the rotation uses one reciprocal square root of f^2 + g^2 (in place
        // of hypot and a division): float64 issue slots are scarce on GB300.
        const double rr = fma(f, f, g * g);
        if (rr == 0.0) {  // split: recover and restart the sweep
          E_(i + 1) = 0.0;
          D_(i + 1) = d_up - shift_acc;
          Z_(i + 1) = z_up;
          E_(m) = 0.0;
          deflated = true;
          break;
        }
        const double rinv = rsqrt(rr);
        r = rr * rinv;
        E_(i + 1) = r;
        s = f * rinv;
        c = g * rinv;
        g = d_up - shift_acc;
        r = (d_i - g) * s + 2.0 * c * bb;
        shift_acc = s * r;
        D_(i + 1) = g + shift_acc;
        g = c * r - bb;
        Z_(i + 1) = s * z_i + c * z_up;
        z_up = c * z_i - s * z_up;  // the new z_i, input of the next rotation
        d_up = d_i;
        e_i = e_nx;
        d_i = d_nx;
        z_i = z_nx;
      }
      if (deflated) continue;
      Z_(l) = z_up;
      D_(l) -= shift_acc;
      E_(l) = g;
      E_(m) = 0.0;
    }
  }
  // ascending order (insertion sort of (lambda, s_1^2) pairs), as eigh returns
  for (int i = 0; i < k; ++i) Z_(i) = Z_(i) * Z_(i);
  for (int i = 1; i < k; ++i) {
    const double dv = D_(i), zv = Z_(i);
    int j = i - 1;
    while (j >= 0 && D_(j) > dv) {
      D_(j + 1) = D_(j);
      Z_(j + 1) = Z_(j);
      --j;
    }
    D_(j + 1) = dv;
    Z_(j + 1) = zv;
  }
  double acc = 0.0;
  for (int i = 0; i < k; ++i) {
    const double lam = D_(i);
    double fl;
    if (fun == MFG_FUN_LOG)
      fl = log(lam);
    else if (fun == MFG_FUN_EXP)
      fl = exp(param * lam);
    else if (fun == MFG_FUN_POW)
      fl = pow(lam, param);
    else
      fl = 0.0;
    acc += fl * Z_(i);
    if (eigvals) eigvals[(size_t)b * k + i] = lam;
    if (first_sq) first_sq[(size_t)b * k + i] = Z_(i);
  }
  if (!ok) {
    acc = nan("");
    if (status) atomicExch(status, (int)MFG_ERR_NO_CONVERGENCE);
  }
  if (values) values[b] = (scale ? scale[b] : 1.0) * acc;
#undef D_
#undef E_
#undef Z_
}

int launch_tridiag_quadrature(int64_t k, int64_t p, const double *H, int32_t fun, double param,
                              const double *scale, double *values, double *eigvals,
                              double *first_sq, int *status, cudaStream_t s) {
  if (p <= 0 || k <= 0) return MFG_OK;
  const size_t per_thread = (size_t)3 * k * sizeof(double);
  const size_t budget = 46 * 1024;  // under the default dynamic shared-memory limit
  if (per_thread > budget) return MFG_ERR_UNSUPPORTED;
  // The solve is a serial float64 chain per problem: spread the problems over
  // all SMs (a few threads per CTA) so that no SM's float64 pipe is shared
  // by many of them.
  int sms = 152;
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int tb = 1;
  while (tb < 32 && (int64_t)tb * sms < p) tb <<= 1;
  while (tb > 1 && (size_t)tb * per_thread > budget) tb >>= 1;
  const unsigned grid = (unsigned)ceil_div(p, tb);
  tridiag_ql_kernel<<<grid, tb, (size_t)tb * per_thread, s>>>((int)k, p, H, fun, param, scale,
                                                              values, eigvals, first_sq, status);
  return MFG_LAUNCH_STATUS();
}

// mean and standard error (population std / sqrt(p)) of p values; one CTA.
__global__ void mean_sem_kernel(const double *__restrict__ v, int64_t p, double *__restrict__ out) {
  __shared__ double red[kWarps];
  __shared__ double s_mean;
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < p; i += blockDim.x) acc += v[i];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < kWarps; ++q) t += red[q];
    s_mean = t / (double)p;
  }
  __syncthreads();
  const double mean = s_mean;
  double sq = 0.0;
  for (int64_t i = threadIdx.x; i < p; i += blockDim.x) {
    const double dv = v[i] - mean;
    sq += dv * dv;
  }
  sq = warp_sum(sq);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < kWarps; ++q) t += red[q];
    out[0] = mean;
    out[1] = sqrt(t / (double)p) / sqrt((double)p);
  }
}

int launch_mean_sem(const double *values, int64_t p, double *mean_sem, cudaStream_t s) {
  if (p <= 0) return MFG_ERR_BAD_ARG;
  mean_sem_kernel<<<1, kThreads, 0, s>>>(values, p, mean_sem);
  return MFG_LAUNCH_STATUS();
}

}  // namespace mfg
