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

// ------------------------------------------------- full eigenvectors, warp per problem
//
// Eigenvalues (ascending) and the full eigenvector matrix of each T, for the
// derivative of e1^T f(T) e1 (the Daleckii-Krein form needs every
// eigenvector).  Implicit QL with Wilkinson shifts as above.  Lane 0 runs
// each sweep's shift chase alone (inputs loaded one rotation ahead, as in the
// first-row kernel) and records the rotations; the warp then applies them,
// in order, to its rows of Z (rows lane, lane + 32, ...).  Z (scratch) is
// row-major k x k; the sorted eigenvectors go to S as columns
// (S[r][j] = component r of vector j).

__global__ void tridiag_eigh_full_kernel(int k, int64_t p, const double *__restrict__ H,
                                         double *__restrict__ w_out, double *__restrict__ S,
                                         double *__restrict__ Z, int *__restrict__ status) {
  extern __shared__ double smf[];
  const int lane = threadIdx.x & 31;
  const int64_t b = blockIdx.x;
  if (b >= p) return;
  double *d = smf;
  double *e = d + k;
  double *rc = e + k;   // rotation i of the current sweep: cosine
  double *rs = rc + k;  // and sine
  int *perm = reinterpret_cast<int *>(rs + k);
  const double *Hb = H + (size_t)b * k * k;
  double *Zb = Z + (size_t)b * k * k;
  for (int i = lane; i < k; i += 32) {
    d[i] = Hb[(size_t)i * k + i];
    e[i] = (i + 1 < k) ? 0.5 * (Hb[(size_t)i * k + i + 1] + Hb[(size_t)(i + 1) * k + i]) : 0.0;
  }
  for (int r = lane; r < k; r += 32)
    for (int c = 0; c < k; ++c) Zb[(size_t)r * k + c] = r == c ? 1.0 : 0.0;
  __syncwarp();
  int ok = 1;
  for (int l = 0; l < k; ++l) {
    int sweeps = 0;
    while (true) {
      // lane 0: one sweep of the chase; the rotations applied are i = hi_i
      // down to lo_i (none when l has converged, or on failure)
      int hi_i = -1, lo_i = 0, done = 0;
      if (lane == 0) {
        int m = l;
        for (; m < k - 1; ++m) {
          const double dd = fabs(d[m]) + fabs(d[m + 1]);
          if (fabs(e[m]) <= DBL_EPSILON * dd) break;
        }
        if (m == l) {
          done = 1;
        } else if (++sweeps > kMaxSweeps) {
          done = 1;
          ok = 0;
        } else {
          double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
          double r = hypot(g, 1.0);
          g = d[m] - d[l] + e[l] / (g + copysign(r, g));
          double sn = 1.0, cs = 1.0, shift_acc = 0.0;
          bool deflated = false;
          double d_up = d[m];
          double e_i = e[m - 1], d_i = d[m - 1];
          hi_i = m - 1;
          lo_i = m;  // the last rotation applied so far
          for (int i = m - 1; i >= l; --i) {
            double e_nx = 0.0, d_nx = 0.0;
            if (i > l) {
              e_nx = e[i - 1];
              d_nx = d[i - 1];
            }
            const double f = sn * e_i;
            const double bb = cs * e_i;
            const double rr = fma(f, f, g * g);
            if (rr == 0.0) {  // split: recover and restart the sweep
              e[i + 1] = 0.0;
              d[i + 1] = d_up - shift_acc;
              e[m] = 0.0;
              deflated = true;
              break;
            }
            const double rinv = rsqrt(rr);
            e[i + 1] = rr * rinv;
            sn = f * rinv;
            cs = g * rinv;
            g = d_up - shift_acc;
            r = (d_i - g) * sn + 2.0 * cs * bb;
            shift_acc = sn * r;
            d[i + 1] = g + shift_acc;
            g = cs * r - bb;
            rc[i] = cs;
            rs[i] = sn;
            lo_i = i;
            d_up = d_i;
            e_i = e_nx;
            d_i = d_nx;
          }
          if (!deflated) {
            d[l] -= shift_acc;
            e[l] = g;
            e[m] = 0.0;
          }
        }
      }
      done = __shfl_sync(0xffffffffu, done, 0);
      hi_i = __shfl_sync(0xffffffffu, hi_i, 0);
      lo_i = __shfl_sync(0xffffffffu, lo_i, 0);
      __syncwarp();  // rc, rs written by lane 0
      if (done) break;
      // the sweep's rotations on columns (i, i + 1) of this lane's rows of Z
      for (int row = lane; row < k; row += 32) {
        double *zr = Zb + (size_t)row * k;
        double zu = zr[hi_i + 1];
        for (int i = hi_i; i >= lo_i; --i) {
          const double zi = zr[i];
          zr[i + 1] = rs[i] * zi + rc[i] * zu;
          zu = rc[i] * zi - rs[i] * zu;
        }
        zr[lo_i] = zu;
      }
      __syncwarp();
    }
    ok = __shfl_sync(0xffffffffu, ok, 0);
    if (!ok) break;
  }
  // ascending order: permutation by insertion sort (lane 0), then a gather of
  // the columns into S
  if (lane == 0) {
    for (int i = 0; i < k; ++i) perm[i] = i;
    for (int i = 1; i < k; ++i) {
      const int pi = perm[i];
      const double dv = d[pi];
      int j = i - 1;
      while (j >= 0 && d[perm[j]] > dv) {
        perm[j + 1] = perm[j];
        --j;
      }
      perm[j + 1] = pi;
    }
  }
  __syncwarp();
  double *Sb = S + (size_t)b * k * k;
  for (int j = lane; j < k; j += 32) w_out[(size_t)b * k + j] = ok ? d[perm[j]] : nan("");
  for (int row = lane; row < k; row += 32)
    for (int j = 0; j < k; ++j) Sb[(size_t)row * k + j] = Zb[(size_t)row * k + perm[j]];
  if (!ok && lane == 0 && status) atomicExch(status, (int)MFG_ERR_NO_CONVERGENCE);
}

static int launch_tridiag_eigh_ql(int64_t k, int64_t p, const double *H, double *w, double *S,
                                  double *Z, int *status, cudaStream_t s) {
  const size_t smem = (size_t)4 * k * sizeof(double) + (size_t)k * sizeof(int);
  if (smem > 48 * 1024) return MFG_ERR_UNSUPPORTED;
  tridiag_eigh_full_kernel<<<(unsigned)p, 32, smem, s>>>((int)k, p, H, w, S, Z, status);
  return MFG_LAUNCH_STATUS();
}

// ------------------------------------------------- divide and conquer, CTA per problem
//
// Cuppen's divide and conquer with every coupling torn: T = diag(T_1, T_2) +
// rho v v^T with v = e_{mid-1} + e_mid, so the leaves are the 1 x 1 blocks
// d_i - e_{i-1} - e_i.  Segments of width w = 1, 2, 4, ... are merged pairwise
// level by level.  A merge of (Q_1, L_1) and (Q_2, L_2) diagonalises
// D + rho z z^T with z = [last row of Q_1; first row of Q_2]; only the first
// and last rows of the eigenvector matrices are carried, because the
// quadrature needs the first row and the next merge needs the last.
//
// Per merge (D sorted, rho made positive by negating the problem):
//  * deflation (Dongarra-Sorensen): rho |z_i| <= tol drops pole i with its
//    unit vector; two kept poles closer than tol are rotated so that one of
//    them drops;
//  * secular roots of 1/rho + sum_i z_i^2 / (d_i - lambda): each root is
//    kept as an offset x from its nearer pole d_o, so that the differences
//    d_i - lambda = (d_i - d_o) - x are accurate.  The iteration interpolates
//    the two poles bounding the root with rational terms, the pole at the
//    origin with its true weight (the fixed-weight scheme of R.-C. Li,
//    "Solving secular equations stably and efficiently", 1993); the largest
//    root uses the two poles below it.  Steps outside the sign bracket fall
//    back to bisection;
//  * z is recomputed from the roots by the Loewner formula (Gu and
//    Eisenstat, 1994), which makes the eigenvectors u_j = zhat / (D - lambda_j)
//    orthogonal to working precision; the new first/last rows are
//    [f; 0]^T u_j and [0; l]^T u_j.
//
// One CTA owns one problem.  The serial parts of a merge (the sorted merge
// of the two halves and the deflation scan) run on one thread per merge; the
// roots, the Loewner products and the vector rows run on one group of lanes
// per root, over all merges of a level at once: one lane for merges of up to
// 16 poles, four lanes (each taking every fourth term of the sums) above.  The float64 work of a problem spreads over up
// to 4k threads in place of the single serial chain of the QL chase; GB300
// issues float64 at two lanes per clock per SM, and the many independent
// chains keep that pipe fed.

constexpr int kDcMinK = 16;          // below this the QL chase is as fast
constexpr int kDcMaxK = 2048;        // shared-memory bound (about 200 KB)
constexpr int kSecularMaxIt = 128;   // bisection alone halves 2^-128 of the bracket
constexpr int kDcMaxThreads = 512;   // at ~120 registers a thread, within an SM's 64K

struct DcLayout {
  int kh;      // merges per level at most
  size_t words;  // 8-byte words per problem
};

__host__ __device__ inline DcLayout dc_layout(int k) {
  DcLayout L;
  L.kh = (k + 1) / 2;
  // LAM FR LR D Z F L X NF NL EO (k each), RH UB (kh each), O (k ints), MS (kh ints)
  L.words = (size_t)11 * k + 2 * (size_t)L.kh + ((size_t)k + L.kh + 1) / 2;
  return L;
}

// root in (P1, P2) of c + s1/(P1 - x) + s2/(P2 - x) = 0, one of P1, P2 zero
__device__ __forceinline__ double dc_quad_root(double c, double P1, double P2, double s1,
                                               double s2) {
  const double a1 = c * (P1 + P2) + s1 + s2;
  const double a0 = c * P1 * P2 + s1 * P2 + s2 * P1;
  // g(x) = c x^2 - a1 x + a0 is positive at P1 and negative at P2, so the
  // root inside is (a1 - sqrt(a1^2 - 4 c a0)) / (2c) for either sign of c
  const double sq = sqrt(fmax(a1 * a1 - 4.0 * c * a0, 0.0));
  return a1 > 0.0 ? 2.0 * a0 / (a1 + sq) : (a1 - sq) / (2.0 * c);
}

// step eta with c + s1/(A - eta) + s2/(B - eta) = 0, A < 0 < B, where the
// model equals f at eta = 0 (so its constant term is A B f)
__device__ __forceinline__ double dc_quad_step(double c, double A, double B, double s1,
                                               double s2, double f) {
  const double a1 = c * (A + B) + s1 + s2;
  const double a0 = A * B * f;
  const double sq = sqrt(fmax(a1 * a1 - 4.0 * c * a0, 0.0));
  return a1 > 0.0 ? 2.0 * a0 / (a1 + sq) : (a1 - sq) / (2.0 * c);
}

// step eta > A with c + s0/(A0 - eta) + s1/(A - eta) = 0, A0 < A < 0 (the
// largest root: both poles below it, so the root is the larger one)
__device__ __forceinline__ double dc_quad_step_right(double c, double A0, double A, double s0,
                                                     double s1, double f) {
  const double a1 = c * (A0 + A) + s0 + s1;
  const double a0 = A0 * A * f;
  const double sq = sqrt(fmax(a1 * a1 - 4.0 * c * a0, 0.0));
  return a1 >= 0.0 ? (a1 + sq) / (2.0 * c) : 2.0 * a0 / (a1 - sq);
}

// 1/x from the hardware's approximate float64 reciprocal (rcp.approx.ftz.f64)
// refined by two Newton-Raphson steps y <- y + y (1 - x y), each of which
// squares the relative error: a few ulp from 1/x for x in the normal range,
// in four FMAs in place of a correctly rounded division.  The secular sums,
// Loewner products and vector entries below carry rounding errors of that
// size anyway.
__device__ __forceinline__ double rcp_nr(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

// Sum (product) over the G lanes of a group (lanes G m .. G m + G - 1 of a
// warp, G = 1 or 4).  Every lane gets the same bits ((v0+v1)+(v2+v3) in some
// operand order; IEEE addition and multiplication commute), so the lanes of a
// group take the same branches afterwards.
template <int G>
__device__ __forceinline__ double group_sum(double v, unsigned mask) {
  if (G >= 2) v += __shfl_xor_sync(mask, v, 1);
  if (G >= 4) v += __shfl_xor_sync(mask, v, 2);
  return v;
}
template <int G>
__device__ __forceinline__ double group_prod(double v, unsigned mask) {
  if (G >= 2) v *= __shfl_xor_sync(mask, v, 1);
  if (G >= 4) v *= __shfl_xor_sync(mask, v, 2);
  return v;
}

// Root j of the secular equation of the kept poles P[0..mk) (ascending) with
// weights ZZ[i] = z_i^2 and coupling rho > 0; upper bounds the largest root.
// The G lanes of a group (sub = 0..G-1, lane mask gm) each sum every G-th
// term and take identical steps.  Every term runs through one loop whose trip
// count is the same for all roots of a merge (the two poles of the model are
// masked out rather than skipped), so the groups of a warp stay converged.
// Returns false when the iteration limit is reached.
template <int G>
__device__ bool dc_secular_root(const double *P, const double *ZZ, int mk, int j, double rho,
                                double upper, int sub, unsigned gm, double &x_out, int &o_out) {
  const double ir = 1.0 / rho;
  const bool last = j + 1 >= mk;
  const double lo_pole = P[j];
  const double hi_pole = last ? upper : P[j + 1];
  const double xma = 0.5 * (lo_pole + hi_pole);
  double fpart = 0.0;
  for (int i = sub; i < mk; i += G) fpart = fma(ZZ[i], rcp_nr(P[i] - xma), fpart);
  const double fmid = ir + group_sum<G>(fpart, gm);
  const double zzj = ZZ[j];
  const double zzj1 = last ? 0.0 : ZZ[j + 1];
  const bool two_below = last && mk > 1;
  const double zzjm = two_below ? ZZ[j - 1] : 0.0;
  const int o = (!last && fmid < 0.0) ? j + 1 : j;
  const double base = P[o];
  double lo = lo_pole - base, hi = hi_pole - base;
  const double P1 = P[j] - base;
  const double P2 = last ? hi : P[j + 1] - base;
  const double P0 = two_below ? P[j - 1] - base : 0.0;
  const double xm = 0.5 * (lo + hi);
  // first guess: the two poles of the model exact, the other terms frozen at
  // the midpoint of the interval
  double x;
  if (mk == 1) {
    x = rho * zzj;
  } else if (last) {
    const double c = fmid - zzj * rcp_nr(P[j] - xma) - zzjm * rcp_nr(P[j - 1] - xma);
    x = c > 0.0 ? xm + dc_quad_step_right(c, P0 - xm, P1 - xm, zzjm, zzj, fmid) : xm;
  } else {
    const double c = fmid - zzj * rcp_nr(P[j] - xma) - zzj1 * rcp_nr(P[j + 1] - xma);
    x = dc_quad_root(c, P1, P2, zzj, zzj1);
  }
  if (!(lo < x && x < hi)) x = xm;
  // the poles of the model: (j, j+1) inside, (j-1, j) for the largest root
  const int m0 = two_below ? j - 1 : j;
  const int m1 = last ? j : j + 1;
  bool conv = false;
  for (int it = 0; it < kSecularMaxIt; ++it) {
    // the rest of the sum (poles below contribute t < 0, above t > 0), its
    // derivative and its absolute sum
    double rs = 0.0, drs = 0.0, ab = 0.0;
    for (int i = sub; i < mk; i += G) {
      const double inv = rcp_nr((P[i] - base) - x);
      double t = ZZ[i] * inv;
      t = (i >= m0 && i <= m1) ? 0.0 : t;
      rs += t;
      drs = fma(t, inv, drs);
      ab += fabs(t);
    }
    rs = group_sum<G>(rs, gm);
    drs = group_sum<G>(drs, gm);
    ab = group_sum<G>(ab, gm);
    const double A = P1 - x;
    const double B = P2 - x;
    const double A0 = P0 - x;
    const double tj = zzj * rcp_nr(A);
    const double tj1 = last ? 0.0 : zzj1 * rcp_nr(B);
    const double tjm = two_below ? zzjm * rcp_nr(A0) : 0.0;
    const double f = ir + rs + tj + tj1 + tjm;
    const double sab = ab + fabs(tj) + fabs(tj1) + fabs(tjm);
    if (f > 0.0)
      hi = x;
    else
      lo = x;
    if (fabs(f) <= DBL_EPSILON * mk * (ir + sab) ||
        hi - lo <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi))) {
      conv = true;
      break;
    }
    double eta;
    if (last && mk == 1) {
      eta = A + zzj * rho;
    } else if (last) {
      const double c = ir + rs - drs * A0;
      eta = c > 0.0 ? dc_quad_step_right(c, A0, A, zzjm + drs * A0 * A0, zzj, f) : nan("");
    } else {
      eta = (o == j) ? dc_quad_step(ir + rs - drs * B, A, B, zzj, zzj1 + drs * B * B, f)
                     : dc_quad_step(ir + rs - drs * A, A, B, zzj + drs * A * A, zzj1, f);
    }
    if (fabs(eta) <= 2.0 * DBL_EPSILON * fabs(x)) {
      conv = true;
      break;
    }
    double xn = x + eta;
    if (!(lo < xn && xn < hi)) xn = 0.5 * (lo + hi);  // also catches a NaN step
    x = xn;
  }
  x_out = x;
  o_out = o;
  return conv;
}

struct DcArrays {
  double *D, *Z, *F, *L, *X, *NF, *NL, *RH, *UB;
  int *O, *MS;
};
constexpr int kFlipBit = 1 << 30;   // in MS: the merge was negated
constexpr int kDcNarrow = 16;       // merges up to this size: one lane per root

// Phases B-D of one level (merges of width 2^(s+1)): the secular roots, the
// Loewner zhat and the new first/last rows, one group of G lanes per root.
// kVec: instead of new first/last rows, the normalised coefficients u of
// each root's vector in the kept poles' columns, U[r * k + i] (r the root's
// index in the problem, i < mk).
template <int G, bool kVec = false>
__device__ bool dc_merge_roots(const DcArrays &Ar, int k, int s, int nm, double *U = nullptr) {
  double *D = Ar.D, *Z = Ar.Z, *F = Ar.F, *L = Ar.L, *X = Ar.X, *NF = Ar.NF, *NL = Ar.NL;
  const double *RH = Ar.RH, *UB = Ar.UB;
  int *O = Ar.O;
  const int *MS = Ar.MS;
  const int tid = threadIdx.x;
  const int sub = tid & (G - 1);
  const int grp = tid / G, ngrp = (int)blockDim.x / G;
  const unsigned gm = (G == 1 ? 1u : (1u << G) - 1u) << (tid & 31 & ~(G - 1));
  bool ok = true;
  // B: secular roots, one group per root over all merges of the level
  for (int r = grp; r < k; r += ngrp) {
    const int q = r >> (s + 1);
    if (q >= nm) continue;
    const int a = q << (s + 1);
    const int j = r - a;
    const int mk = MS[q] & (kFlipBit - 1);
    if (j >= mk) continue;
    double x;
    int o;
    ok &= dc_secular_root<G>(D + a, NF + a, mk, j, RH[q], UB[q], sub, gm, x, o);
    if (sub == 0) {
      X[r] = x;
      O[r] = o;
    }
  }
  __syncthreads();
  // C: Loewner zhat_i^2 = prod_j (lambda_j - d_i) / prod_{j != i} (d_j - d_i) / rho,
  // numerators paired with denominators to stay in range
  for (int r = grp; r < k; r += ngrp) {
    const int q = r >> (s + 1);
    if (q >= nm) continue;
    const int a = q << (s + 1);
    const int i = r - a;
    const int mk = MS[q] & (kFlipBit - 1);
    if (i >= mk) continue;
    const double *P = D + a;
    const double di = P[i];
    double prod = sub == 0 ? ((P[O[a + mk - 1]] - di) + X[a + mk - 1]) / RH[q] : 1.0;
    for (int j = sub; j < mk - 1; j += G)
      prod *= ((P[O[a + j]] - di) + X[a + j]) * rcp_nr(P[j < i ? j : j + 1] - di);
    prod = group_prod<G>(prod, gm);
    if (sub == 0) Z[r] = copysign(sqrt(fmax(prod, 0.0)), Z[r]);
  }
  __syncthreads();
  // D: first/last rows of the merged eigenvectors
  for (int r = grp; r < k; r += ngrp) {
    const int q = r >> (s + 1);
    if (q >= nm) continue;
    const int a = q << (s + 1);
    const int j = r - a;
    const int mk = MS[q] & (kFlipBit - 1);
    if (j >= mk) continue;
    const double *P = D + a;
    const double ox = P[O[r]], x = X[r];
    double s2 = 0.0, sf = 0.0, sl = 0.0;
    for (int i = sub; i < mk; i += G) {
      const double u = Z[a + i] * rcp_nr((P[i] - ox) - x);
      s2 = fma(u, u, s2);
      if (!kVec) {
        sf = fma(F[a + i], u, sf);
        sl = fma(L[a + i], u, sl);
      }
    }
    s2 = group_sum<G>(s2, gm);  // in every lane of the group
    const double rn = rsqrt(s2);
    if (kVec) {
      for (int i = sub; i < mk; i += G)
        U[(size_t)r * k + i] = Z[a + i] * rcp_nr((P[i] - ox) - x) * rn;
    } else {
      sf = group_sum<G>(sf, gm);
      sl = group_sum<G>(sl, gm);
    }
    if (sub == 0) {
      if (!kVec) {
        NF[r] = sf * rn;
        NL[r] = sl * rn;
      }
      X[r] = ox + x;
    }
  }
  __syncthreads();
  return ok;
}

__global__ void __launch_bounds__(kDcMaxThreads, 1)
    tridiag_dc_kernel(int k, int64_t p, const double *__restrict__ H, int fun, double param,
                      const double *__restrict__ scale, double *__restrict__ values,
                      double *__restrict__ eigvals, double *__restrict__ first_sq,
                      int *__restrict__ status) {
  extern __shared__ double sm[];
  const int tid = threadIdx.x;
  const int nt = blockDim.x;
  const int64_t b = blockIdx.x;
  const DcLayout Ly = dc_layout(k);
  double *LAM = sm;       // segment eigenvalues
  double *FR = LAM + k;   // first rows of the segment eigenvector matrices
  double *LR = FR + k;    // last rows
  double *D = LR + k;     // merge: poles (kept first, deflated after)
  double *Z = D + k;      // merge: z, then zhat
  double *F = Z + k;      // merge: first-row entries aligned with D
  double *L = F + k;      // merge: last-row entries aligned with D
  double *X = L + k;      // merge: root offsets, then roots
  double *NF = X + k;     // merge: z^2 of the kept poles, then new first rows
  double *NL = NF + k;    // merge: new last rows
  double *EO = NL + k;    // off-diagonal of T
  double *RH = EO + k;    // per merge: |rho|
  double *UB = RH + Ly.kh;  // per merge: bound of the largest root
  int *O = reinterpret_cast<int *>(UB + Ly.kh);  // per root: origin pole
  int *MS = O + k;        // per merge: kept count and kFlipBit
  const DcArrays Ar{D, Z, F, L, X, NF, NL, RH, UB, O, MS};

  const double *Hb = H + (size_t)b * k * k;
  for (int i = tid; i < k; i += nt)
    EO[i] = (i + 1 < k) ? 0.5 * (Hb[(size_t)i * k + i + 1] + Hb[(size_t)(i + 1) * k + i]) : 0.0;
  __syncthreads();
  for (int i = tid; i < k; i += nt) {
    LAM[i] = Hb[(size_t)i * k + i] - (i > 0 ? EO[i - 1] : 0.0) - EO[i];
    FR[i] = 1.0;
    LR[i] = 1.0;
  }
  __syncthreads();
  bool ok = true;
  for (int s = 0; (1 << s) < k; ++s) {
    const int w = 1 << s;
    const int nm = (k - w - 1) / (2 * w) + 1;
    // A: sorted merge of the two halves and deflation, one thread per merge
    for (int q = tid; q < nm; q += nt) {
      const int a = q * 2 * w, mid = a + w, hi = min(a + 2 * w, k);
      double rho = EO[mid - 1];
      const bool flip = rho < 0.0;
      const double sg = flip ? -1.0 : 1.0;
      rho = fabs(rho);
      const double maxabs = fmax(fmax(fabs(LAM[a]), fabs(LAM[mid - 1])),
                                 fmax(fabs(LAM[mid]), fabs(LAM[hi - 1])));
      const double tol = 8.0 * DBL_EPSILON * fmax(maxabs, 2.0 * rho);
      const int n1 = mid - a, n2 = hi - mid;
      int c1 = 0, c2 = 0, kp = a, dp = hi;
      double zs = 0.0;
      for (int t = a; t < hi; ++t) {
        bool take1;
        if (c1 == n1)
          take1 = false;
        else if (c2 == n2)
          take1 = true;
        else
          take1 = sg * LAM[flip ? mid - 1 - c1 : a + c1] <= sg * LAM[flip ? hi - 1 - c2 : mid + c2];
        double d, z, f, l;
        if (take1) {
          const int i1 = flip ? mid - 1 - c1 : a + c1;
          d = sg * LAM[i1];
          z = LR[i1];
          f = FR[i1];
          l = 0.0;
          ++c1;
        } else {
          const int i2 = flip ? hi - 1 - c2 : mid + c2;
          d = sg * LAM[i2];
          z = FR[i2];
          f = 0.0;
          l = LR[i2];
          ++c2;
        }
        if (rho * fabs(z) <= tol) {  // negligible coupling: d is an eigenvalue
          --dp;
          D[dp] = d;
          F[dp] = f;
          L[dp] = l;
          continue;
        }
        zs = fma(z, z, zs);
        if (kp > a && d - D[kp - 1] <= tol) {
          // two poles closer than tol: rotate the weight of the earlier one
          // onto this one and drop the earlier one
          const double zp = Z[kp - 1];
          const double r = hypot(zp, z);
          const double c = z / r, sn = zp / r;
          const double fp = F[kp - 1], lp = L[kp - 1];
          --dp;
          D[dp] = D[kp - 1];
          F[dp] = c * fp - sn * f;
          L[dp] = c * lp - sn * l;
          D[kp - 1] = d;
          Z[kp - 1] = r;
          NF[kp - 1] = r * r;
          F[kp - 1] = sn * fp + c * f;
          L[kp - 1] = sn * lp + c * l;
        } else {
          D[kp] = d;
          Z[kp] = z;
          NF[kp] = z * z;
          F[kp] = f;
          L[kp] = l;
          ++kp;
        }
      }
      // the dropped poles sit in [dp, hi) in reverse push order, ascending
      // except for rotated ones: reverse, then insertion-sort the short run
      for (int u = dp, v = hi - 1; u < v; ++u, --v) {
        double tmp = D[u]; D[u] = D[v]; D[v] = tmp;
        tmp = F[u]; F[u] = F[v]; F[v] = tmp;
        tmp = L[u]; L[u] = L[v]; L[v] = tmp;
      }
      for (int u = dp + 1; u < hi; ++u) {
        const double dv = D[u], fv = F[u], lv = L[u];
        int v = u - 1;
        while (v >= dp && D[v] > dv) {
          D[v + 1] = D[v];
          F[v + 1] = F[v];
          L[v + 1] = L[v];
          --v;
        }
        D[v + 1] = dv;
        F[v + 1] = fv;
        L[v + 1] = lv;
      }
      const int mk = kp - a;
      MS[q] = mk | (flip ? kFlipBit : 0);
      RH[q] = rho;
      // the largest root lies below d_max + rho |z|^2; the margin keeps it
      // strictly inside when a single pole is kept
      UB[q] = mk > 0 ? D[kp - 1] + rho * zs * (1.0 + 16.0 * DBL_EPSILON) +
                           16.0 * DBL_EPSILON * fabs(D[kp - 1])
                     : 0.0;
    }
    __syncthreads();
    ok &= (2 << s) > kDcNarrow ? dc_merge_roots<4>(Ar, k, s, nm) : dc_merge_roots<1>(Ar, k, s, nm);
    // E: merge the roots [a, a+mk) with the dropped poles [a+mk, hi), both
    // ascending; a negated merge is negated back and reversed
    for (int q = tid; q < nm; q += nt) {
      const int a = q * 2 * w, hi = min(a + 2 * w, k);
      const int mk = MS[q] & (kFlipBit - 1);
      const bool flip = (MS[q] & kFlipBit) != 0;
      const double sg = flip ? -1.0 : 1.0;
      int c1 = a, c2 = a + mk;
      for (int t = 0; t < hi - a; ++t) {
        double v, fv, lv;
        if (c1 < a + mk && (c2 >= hi || X[c1] <= D[c2])) {
          v = X[c1];
          fv = NF[c1];
          lv = NL[c1];
          ++c1;
        } else {
          v = D[c2];
          fv = F[c2];
          lv = L[c2];
          ++c2;
        }
        const int pos = flip ? hi - 1 - t : a + t;
        LAM[pos] = sg * v;
        FR[pos] = fv;
        LR[pos] = lv;
      }
    }
    __syncthreads();
  }
  ok = __syncthreads_and(ok) != 0;
  double acc = 0.0;
  for (int i = tid; i < k; i += nt) {
    const double lam = LAM[i];
    const double w2 = FR[i] * FR[i];
    double fl;
    if (fun == MFG_FUN_LOG)
      fl = log(lam);
    else if (fun == MFG_FUN_EXP)
      fl = exp(param * lam);
    else if (fun == MFG_FUN_POW)
      fl = pow(lam, param);
    else
      fl = 0.0;
    acc = fma(fl, w2, acc);
    if (eigvals) eigvals[(size_t)b * k + i] = lam;
    if (first_sq) first_sq[(size_t)b * k + i] = w2;
  }
  // fixed-order CTA sum: warp butterflies, then warp partials in order
  __shared__ double red[32];
  acc = warp_sum(acc);
  if ((tid & 31) == 0) red[tid >> 5] = acc;
  __syncthreads();
  if (tid == 0) {
    acc = 0.0;
    for (int w = 0; w < (nt >> 5); ++w) acc += red[w];
    if (!ok) {
      acc = nan("");
      if (status) atomicExch(status, (int)MFG_ERR_NO_CONVERGENCE);
    }
    if (values) values[b] = (scale ? scale[b] : 1.0) * acc;
  }
}

// ---------------------------------------- divide and conquer with eigenvectors
//
// The levels, deflation, secular roots and Loewner vectors of
// tridiag_dc_kernel, carrying every eigenvector column (rows a..hi-1 of its
// merge; zero elsewhere) in shared memory instead of first and last rows.
// S, S2 and U are k x k, column c of S at S[c * k].
//   A (one thread per merge): sorted merge of the halves with deflation; each
//     pole keeps the index CI of its column in S (z is that column's entry in
//     row mid-1 or mid), and a close-pole rotation combines two columns in
//     place;
//   B, C, D: dc_merge_roots<G, true>, which leaves each root's normalised
//     coefficients in U;
//   D' (all threads over (column, row) pairs): S2[:, a+j] = S[:, CI[a..a+mk)]
//     U[a+j, :] for the roots, and S2[:, c] = S[:, CI[c]] for the deflated
//     poles c >= a+mk;
//   E: the order of the merged eigenvalues as a column map (in O), then S
//     from S2 through that map.
// A direct restatement runs on the CPU as dc_full in the tests.
constexpr int kDcvMaxK = 64;  // S, S2, U: 3 k^2 doubles (96 KB at k = 64)

__host__ inline size_t dcv_smem_bytes(int k) {
  return (dc_layout(k).words + (size_t)3 * k * k + ((size_t)k + 1) / 2) * sizeof(double);
}

__global__ void __launch_bounds__(kDcMaxThreads, 1)
    tridiag_dcv_kernel(int k, int64_t p, const double *__restrict__ H, double *__restrict__ w_out,
                       double *__restrict__ S_out, int *__restrict__ status) {
  extern __shared__ double sm[];
  const int tid = threadIdx.x;
  const int nt = blockDim.x;
  const int64_t b = blockIdx.x;
  const DcLayout Ly = dc_layout(k);
  double *LAM = sm;
  double *FR = LAM + k;  // unused here (same layout as tridiag_dc_kernel)
  double *LR = FR + k;
  double *D = LR + k;
  double *Z = D + k;
  double *F = Z + k;
  double *L = F + k;
  double *X = L + k;
  double *NF = X + k;
  double *NL = NF + k;
  double *EO = NL + k;
  double *RH = EO + k;
  double *UB = RH + Ly.kh;
  int *O = reinterpret_cast<int *>(UB + Ly.kh);
  int *MS = O + k;
  double *S = sm + Ly.words;
  double *S2 = S + (size_t)k * k;
  double *U = S2 + (size_t)k * k;
  int *CI = reinterpret_cast<int *>(U + (size_t)k * k);
  const DcArrays Ar{D, Z, F, L, X, NF, NL, RH, UB, O, MS};

  const double *Hb = H + (size_t)b * k * k;
  for (int i = tid; i < k; i += nt)
    EO[i] = (i + 1 < k) ? 0.5 * (Hb[(size_t)i * k + i + 1] + Hb[(size_t)(i + 1) * k + i]) : 0.0;
  __syncthreads();
  for (int i = tid; i < k; i += nt) LAM[i] = Hb[(size_t)i * k + i] - (i > 0 ? EO[i - 1] : 0.0) - EO[i];
  for (int idx = tid; idx < k * k; idx += nt) S[idx] = (idx / k == idx % k) ? 1.0 : 0.0;
  __syncthreads();
  bool ok = true;
  for (int s = 0; (1 << s) < k; ++s) {
    const int w = 1 << s;
    const int span = 2 * w;
    const int nm = (k - w - 1) / span + 1;
    // A
    for (int q = tid; q < nm; q += nt) {
      const int a = q * span, mid = a + w, hi = min(a + span, k);
      double rho = EO[mid - 1];
      const bool flip = rho < 0.0;
      const double sg = flip ? -1.0 : 1.0;
      rho = fabs(rho);
      const double maxabs = fmax(fmax(fabs(LAM[a]), fabs(LAM[mid - 1])),
                                 fmax(fabs(LAM[mid]), fabs(LAM[hi - 1])));
      const double tol = 8.0 * DBL_EPSILON * fmax(maxabs, 2.0 * rho);
      const int n1 = mid - a, n2 = hi - mid;
      int c1 = 0, c2 = 0, kp = a, dp = hi;
      double zs = 0.0;
      for (int t = a; t < hi; ++t) {
        bool take1;
        if (c1 == n1)
          take1 = false;
        else if (c2 == n2)
          take1 = true;
        else
          take1 = sg * LAM[flip ? mid - 1 - c1 : a + c1] <= sg * LAM[flip ? hi - 1 - c2 : mid + c2];
        double d, z;
        int col;
        if (take1) {
          col = flip ? mid - 1 - c1 : a + c1;
          z = S[(size_t)col * k + (mid - 1)];  // last row of the upper block
          ++c1;
        } else {
          col = flip ? hi - 1 - c2 : mid + c2;
          z = S[(size_t)col * k + mid];  // first row of the lower block
          ++c2;
        }
        d = sg * LAM[col];
        if (rho * fabs(z) <= tol) {
          --dp;
          D[dp] = d;
          CI[dp] = col;
          continue;
        }
        zs = fma(z, z, zs);
        if (kp > a && d - D[kp - 1] <= tol) {
          // close poles: the dropped column is c Vprev - sn Vcur (in column
          // cp), the kept one sn Vprev + c Vcur (in column col)
          const double zp = Z[kp - 1];
          const double r = hypot(zp, z);
          const double c = z / r, sn = zp / r;
          const int cp = CI[kp - 1];
          for (int t2 = a; t2 < hi; ++t2) {
            const double vp = S[(size_t)cp * k + t2], vc = S[(size_t)col * k + t2];
            S[(size_t)cp * k + t2] = c * vp - sn * vc;
            S[(size_t)col * k + t2] = sn * vp + c * vc;
          }
          --dp;
          D[dp] = D[kp - 1];
          CI[dp] = cp;
          D[kp - 1] = d;
          Z[kp - 1] = r;
          NF[kp - 1] = r * r;
          CI[kp - 1] = col;
        } else {
          D[kp] = d;
          Z[kp] = z;
          NF[kp] = z * z;
          CI[kp] = col;
          ++kp;
        }
      }
      for (int u = dp, v = hi - 1; u < v; ++u, --v) {
        const double tmp = D[u];
        D[u] = D[v];
        D[v] = tmp;
        const int ti = CI[u];
        CI[u] = CI[v];
        CI[v] = ti;
      }
      for (int u = dp + 1; u < hi; ++u) {
        const double dv = D[u];
        const int cv = CI[u];
        int v = u - 1;
        while (v >= dp && D[v] > dv) {
          D[v + 1] = D[v];
          CI[v + 1] = CI[v];
          --v;
        }
        D[v + 1] = dv;
        CI[v + 1] = cv;
      }
      const int mk = kp - a;
      MS[q] = mk | (flip ? kFlipBit : 0);
      RH[q] = rho;
      UB[q] = mk > 0 ? D[kp - 1] + rho * zs * (1.0 + 16.0 * DBL_EPSILON) +
                           16.0 * DBL_EPSILON * fabs(D[kp - 1])
                     : 0.0;
    }
    __syncthreads();
    ok &= span > kDcNarrow ? dc_merge_roots<4, true>(Ar, k, s, nm, U)
                           : dc_merge_roots<1, true>(Ar, k, s, nm, U);
    // D': the merged columns into S2 (rows a..hi-1)
    for (int idx = tid; idx < nm * span * span; idx += nt) {
      const int q = idx / (span * span);
      const int rem = idx - q * span * span;
      const int j = rem / span, tt = rem - j * span;
      const int a = q * span, hi = min(a + span, k);
      const int c = a + j, t = a + tt;
      if (c >= hi || t >= hi) continue;
      const int mk = MS[q] & (kFlipBit - 1);
      if (j < mk) {
        const double *u = U + (size_t)c * k;
        double acc = 0.0;
        for (int i = 0; i < mk; ++i) acc = fma(u[i], S[(size_t)CI[a + i] * k + t], acc);
        S2[(size_t)c * k + t] = acc;
      } else {
        S2[(size_t)c * k + t] = S[(size_t)CI[c] * k + t];
      }
    }
    // E: ascending merge of the roots [a, a+mk) and the dropped poles
    // [a+mk, hi); a negated merge is negated back and reversed
    for (int q = tid; q < nm; q += nt) {
      const int a = q * span, hi = min(a + span, k);
      const int mk = MS[q] & (kFlipBit - 1);
      const bool flip = (MS[q] & kFlipBit) != 0;
      const double sg = flip ? -1.0 : 1.0;
      int c1 = a, c2 = a + mk;
      for (int t = 0; t < hi - a; ++t) {
        double v;
        int src;
        if (c1 < a + mk && (c2 >= hi || X[c1] <= D[c2])) {
          v = X[c1];
          src = c1++;
        } else {
          v = D[c2];
          src = c2++;
        }
        const int pos = flip ? hi - 1 - t : a + t;
        LAM[pos] = sg * v;
        O[pos] = src;
      }
    }
    __syncthreads();
    for (int idx = tid; idx < nm * span * span; idx += nt) {
      const int q = idx / (span * span);
      const int rem = idx - q * span * span;
      const int j = rem / span, tt = rem - j * span;
      const int a = q * span, hi = min(a + span, k);
      const int c = a + j, t = a + tt;
      if (c >= hi || t >= hi) continue;
      S[(size_t)c * k + t] = S2[(size_t)O[c] * k + t];
    }
    __syncthreads();
  }
  ok = __syncthreads_and(ok) != 0;
  for (int j = tid; j < k; j += nt) w_out[(size_t)b * k + j] = ok ? LAM[j] : nan("");
  double *Sb = S_out + (size_t)b * k * k;
  for (int idx = tid; idx < k * k; idx += nt) {
    const int row = idx / k, j = idx - row * k;
    Sb[idx] = S[(size_t)j * k + row];
  }
  if (!ok && tid == 0 && status) atomicExch(status, (int)MFG_ERR_NO_CONVERGENCE);
}

int launch_tridiag_quadrature(int64_t k, int64_t p, const double *H, int32_t fun, double param,
                              const double *scale, double *values, double *eigvals,
                              double *first_sq, int *status, cudaStream_t s) {
  if (p <= 0 || k <= 0) return MFG_OK;
  if (k >= kDcMinK && k <= kDcMaxK) {
    // one problem per CTA, a quad of lanes per root: 4k threads up to 512
    const size_t smem = dc_layout((int)k).words * sizeof(double);
    if (smem > 48 * 1024)
      MFG_CUDA_TRY(cudaFuncSetAttribute(tridiag_dc_kernel,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int threads = (int)(k >= kDcMaxThreads / 4 ? kDcMaxThreads : (4 * k + 31) / 32 * 32);
    tridiag_dc_kernel<<<(unsigned)p, threads, smem, s>>>((int)k, p, H, fun, param, scale, values,
                                                        eigvals, first_sq, status);
    return MFG_LAUNCH_STATUS();
  }
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

// Every eigenvector: divide and conquer for kDcMinK <= k <= kDcvMaxK (the
// gradient's k), implicit QL otherwise.
int launch_tridiag_eigh_full(int64_t k, int64_t p, const double *H, double *w, double *S,
                             double *Z, int *status, cudaStream_t s) {
  if (p <= 0 || k <= 0) return MFG_OK;
  if (k >= kDcMinK && k <= kDcvMaxK) {
    const size_t smem = dcv_smem_bytes((int)k);
    MFG_CUDA_TRY(cudaFuncSetAttribute(tridiag_dcv_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int threads = (int)((4 * k + 31) / 32 * 32);
    tridiag_dcv_kernel<<<(unsigned)p, threads, smem, s>>>((int)k, p, H, w, S, status);
    return MFG_LAUNCH_STATUS();
  }
  return launch_tridiag_eigh_ql(k, p, H, w, S, Z, status, s);
}

}  // namespace mfg
