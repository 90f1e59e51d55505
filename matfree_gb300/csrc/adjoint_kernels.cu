// Small float64 kernels of the batched Hessenberg adjoint (reverse Arnoldi).
//
// The reverse sweep keeps, per probe b, the k x k matrices Gamma and
// Pi_gamma = H dH^T - dc c e1 e1^T and a few length-k coefficient vectors.
// These kernels update them between the n-length sweeps (projections,
// updates, operator application) that the driver issues with the forward
// kernels.  Index conventions follow the float64 restatement of
// matfree/decomp.py:480-600: step idx runs from k-1 down to 0.
#include "common.cuh"
#include "kernels.cuh"

namespace mfg {

// Pi[b][i][j] = sum_l H[b][i][l] dH[b][j][l]  - (i == j == 0) dc_b c_b
__global__ void pi_gamma_kernel(const double *__restrict__ H, const double *__restrict__ dH,
                                const double *__restrict__ dc, const double *__restrict__ c,
                                int k, int64_t p, double *__restrict__ Pi) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t kk = (int64_t)k * k;
  if (t >= p * kk) return;
  const int64_t b = t / kk;
  const int i = (int)((t % kk) / k), j = (int)(t % k);
  const double *Hb = H + b * kk, *dHb = dH + b * kk;
  double acc = 0.0;
  for (int l = 0; l < k; ++l) acc += Hb[(int64_t)i * k + l] * dHb[(int64_t)j * k + l];
  if (i == 0 && j == 0 && dc) acc -= dc[b] * c[b];
  Pi[t] = acc;
}

// gamma[b][j] = dH[b][j][k-1] - h[b][j]  (h = Q^T dr, or absent)
// coef[b][j] = -gamma[b][j]               (lambda = dr + Q gamma as an update)
__global__ void adj_init_kernel(const double *__restrict__ dH, const double *__restrict__ h, int k,
                                int64_t p, double *__restrict__ gamma, double *__restrict__ coef) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= p * k) return;
  const int64_t b = t / k;
  const int j = (int)(t % k);
  double g = dH[b * k * k + (int64_t)j * k + (k - 1)];
  if (h) g -= h[t];
  gamma[t] = g;
  coef[t] = -g;
}

// masked re-projection coefficients of step idx:
// coef[b][j] = h[b][j] - dH[b][j][idx] for j < ncols (columns 0..idx+1)
__global__ void adj_reortho_coef_kernel(const double *__restrict__ h, const double *__restrict__ dH,
                                        int k, int64_t p, int idx, int ncols,
                                        double *__restrict__ coef) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= p * ncols) return;
  const int64_t b = t / ncols;
  const int j = (int)(t % ncols);
  coef[b * k + j] = h[b * k + j] - dH[b * k * k + (int64_t)j * k + idx];
}

// Step idx after g = Q^T (A^T lambda) (g[b][j], j <= idx):
//   Gamma[idx][j] = m_j (Pi[idx][j] - g_j),  m_j = 1 (j < idx), 1/2 (j = idx), 0
//   coefG[j] = -(Gamma[idx][j] + Gamma[j][idx])   (xi adds Q (Gamma + Gamma^T)[idx, :])
//   bp[j] = H[idx][j] for j > idx, else 0        (beta_plus row of idx)
//   scal = (alpha = H[idx][idx], gamma_idx, beta_minus = H[idx][idx-1] or 1)
__global__ void adj_step_coef_kernel(const double *__restrict__ H, const double *__restrict__ Pi,
                                     const double *__restrict__ g, const double *__restrict__ gamma,
                                     int k, int64_t p, int idx, double *__restrict__ Gamma,
                                     double *__restrict__ coefG, double *__restrict__ bp,
                                     double *__restrict__ scal) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= p * k) return;
  const int64_t b = t / k;
  const int j = (int)(t % k);
  const int64_t kk = (int64_t)k * k;
  double *Gb = Gamma + b * kk;
  const double mask = j < idx ? 1.0 : (j == idx ? 0.5 : 0.0);
  const double row = (j <= idx) ? mask * (Pi[b * kk + (int64_t)idx * k + j] - g[b * k + j]) : 0.0;
  Gb[(int64_t)idx * k + j] = row;
  const double colv = (j == idx) ? row : Gb[(int64_t)j * k + idx];
  coefG[b * k + j] = -(row + colv);
  bp[b * k + j] = (j > idx) ? H[b * kk + (int64_t)idx * k + j] : 0.0;
  if (j == 0) {
    scal[b * 3 + 0] = H[b * kk + (int64_t)idx * k + idx];
    scal[b * 3 + 1] = gamma[b * k + idx];
    scal[b * 3 + 2] = idx > 0 ? H[b * kk + (int64_t)idx * k + (idx - 1)] : 1.0;
  }
}

// out[b][r] = U[b][r] - alpha_b lam[b][r] + gam_b R[b][r] (+ dq[b][r] when the
// cotangent of the basis is given: its column idx, dq_bstride apart per probe)
template <typename T>
__global__ void adj_lincomb_kernel(const T *__restrict__ U, const T *__restrict__ lam,
                                   const T *__restrict__ R, const T *__restrict__ dq, int64_t dq_bstride,
                                   const double *__restrict__ scal, int64_t n, int64_t ld, int64_t p,
                                   T *__restrict__ out) {
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t b = blockIdx.y;
  if (r >= n || b >= p) return;
  const T alpha = (T)scal[b * 3 + 0], gam = (T)scal[b * 3 + 1];
  const int64_t o = b * ld + r;
  T v = U[o] - alpha * lam[o] + gam * R[o];
  if (dq) v += dq[b * dq_bstride + r];
  out[o] = v;
}

// y[i] += a x[i] (float64)
__global__ void axpy_f64_kernel(double a, const double *__restrict__ x, double *__restrict__ y,
                                int64_t m) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < m) y[i] += a * x[i];
}

// out[b][r] = sum_i coef[b][i] Q[b][i][r] for r < n, 0 for n <= r < ld: the
// back-projection Q^T (f(T) e1) of a batch of Krylov bases (p, k, ld).  The
// coefficients are staged in shared memory kCombineCoef at a time; each
// thread owns one row and sums over i in a fixed order.
constexpr int kCombineCoef = 512;

template <typename T>
__global__ void __launch_bounds__(256)
basis_combine_kernel(const T *__restrict__ Q, int64_t k, int64_t ld, int64_t n,
                     const double *__restrict__ coef, T *__restrict__ out) {
  __shared__ T sc[kCombineCoef];
  const int64_t b = blockIdx.y;
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const T *Qb = Q + b * k * ld;
  T acc = 0;
  for (int64_t i0 = 0; i0 < k; i0 += kCombineCoef) {
    const int m = (int)(k - i0 < kCombineCoef ? k - i0 : kCombineCoef);
    __syncthreads();
    for (int t = threadIdx.x; t < m; t += blockDim.x) sc[t] = (T)coef[b * k + i0 + t];
    __syncthreads();
    if (r < n)
      for (int t = 0; t < m; ++t) acc += sc[t] * Qb[(i0 + t) * ld + r];
  }
  if (r < ld) out[b * ld + r] = r < n ? acc : (T)0;
}

// beta[b] = scal[b][2] (the divisor of step idx), for the normalise kernel
__global__ void adj_beta_kernel(const double *__restrict__ scal, int64_t p, double *__restrict__ beta) {
  const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (b < p) beta[b] = scal[b * 3 + 2];
}

static inline unsigned blocks(int64_t work, int tb) { return (unsigned)ceil_div(work, tb); }

int launch_pi_gamma(const double *H, const double *dH, const double *dc, const double *c, int k,
                    int64_t p, double *Pi, cudaStream_t s) {
  pi_gamma_kernel<<<blocks(p * k * k, 128), 128, 0, s>>>(H, dH, dc, c, k, p, Pi);
  return MFG_LAUNCH_STATUS();
}

int launch_adj_init(const double *dH, const double *h, int k, int64_t p, double *gamma, double *coef,
                    cudaStream_t s) {
  adj_init_kernel<<<blocks(p * k, 128), 128, 0, s>>>(dH, h, k, p, gamma, coef);
  return MFG_LAUNCH_STATUS();
}

int launch_adj_reortho_coef(const double *h, const double *dH, int k, int64_t p, int idx, int ncols,
                            double *coef, cudaStream_t s) {
  adj_reortho_coef_kernel<<<blocks(p * ncols, 128), 128, 0, s>>>(h, dH, k, p, idx, ncols, coef);
  return MFG_LAUNCH_STATUS();
}

int launch_adj_step_coef(const double *H, const double *Pi, const double *g, const double *gamma,
                         int k, int64_t p, int idx, double *Gamma, double *coefG, double *bp,
                         double *scal, double *beta, cudaStream_t s) {
  adj_step_coef_kernel<<<blocks(p * k, 128), 128, 0, s>>>(H, Pi, g, gamma, k, p, idx, Gamma, coefG,
                                                          bp, scal);
  adj_beta_kernel<<<blocks(p, 128), 128, 0, s>>>(scal, p, beta);
  return MFG_LAUNCH_STATUS();
}

template <typename T>
int launch_adj_lincomb(const T *U, const T *lam, const T *R, const T *dq, int64_t dq_bstride,
                       const double *scal, int64_t n, int64_t ld, int64_t p, T *out, cudaStream_t s) {
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  adj_lincomb_kernel<T><<<dim3(blocks(n, 256), (unsigned)p), 256, 0, s>>>(U, lam, R, dq, dq_bstride, scal,
                                                                          n, ld, p, out);
  return MFG_LAUNCH_STATUS();
}
template int launch_adj_lincomb<float>(const float *, const float *, const float *, const float *,
                                       int64_t, const double *, int64_t, int64_t, int64_t, float *,
                                       cudaStream_t);
template int launch_adj_lincomb<double>(const double *, const double *, const double *, const double *,
                                        int64_t, const double *, int64_t, int64_t, int64_t, double *,
                                        cudaStream_t);

template <typename T>
int launch_basis_combine(const T *Q, int64_t k, int64_t ld, int64_t n, int64_t p, const double *coef,
                         T *out, cudaStream_t s) {
  if (p <= 0) return MFG_OK;
  if (p > 65535) return MFG_ERR_UNSUPPORTED;
  basis_combine_kernel<T><<<dim3(blocks(ld, 256), (unsigned)p), 256, 0, s>>>(Q, k, ld, n, coef, out);
  return MFG_LAUNCH_STATUS();
}
template int launch_basis_combine<float>(const float *, int64_t, int64_t, int64_t, int64_t,
                                         const double *, float *, cudaStream_t);
template int launch_basis_combine<double>(const double *, int64_t, int64_t, int64_t, int64_t,
                                          const double *, double *, cudaStream_t);

int launch_axpy_f64(double a, const double *x, double *y, int64_t m, cudaStream_t s) {
  if (m <= 0) return MFG_OK;
  axpy_f64_kernel<<<blocks(m, 256), 256, 0, s>>>(a, x, y, m);
  return MFG_LAUNCH_STATUS();
}

}  // namespace mfg
