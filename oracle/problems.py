"""Float64 builders of the synthetic SLQ inputs (oracle; test infrastructure).

* ``hermitian_matrix_from_eigenvalues`` restates matfree/test_util.py:6-16
  (Q from a reduced QR of a Gaussian matrix, A = Q diag(eig) Q^T) with a NumPy
  generator in place of a JAX key.
* ``make_A_logdet`` restates the spectrum of
  tests/test_funm/test_monte_carlo_funm_sym_logdet.py:7-13.
* ``dense_spd``: A = B B^T / n + I, B ~ N(0, 1) (the dense float64 workload).
* ``rbf_points``/``rbf_kernel``: x ~ U[0, 1]^3 and
  K = s2 exp(-|x_i - x_j|^2 / (2 l^2)) + tau I.
* ``laplacian_2d``: 5-point Dirichlet stencil on an m x m grid plus shift * I,
  as scipy CSR (int32 indices, float32 values), rows in lexicographic order.
"""

from __future__ import annotations

import concurrent.futures as cf
import os

import numpy as np
import scipy.sparse as sp


def hermitian_matrix_from_eigenvalues(eigvals, rng):
    n = len(eigvals)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    return (Q * np.asarray(eigvals, dtype=np.float64)) @ Q.T


def make_A_logdet(n, num_significant_eigvals, rng):
    d = np.arange(n) / n + 1.0
    d[num_significant_eigvals:] = 0.001
    return hermitian_matrix_from_eigenvalues(d, rng)


def dense_spd(n, seed=0):
    B = np.random.default_rng(seed).standard_normal((n, n))
    return B @ B.T / n + np.eye(n)


def rbf_points(n, seed=0, dim=3):
    return np.random.default_rng(seed).uniform(0.0, 1.0, size=(n, dim))


def row_blocks(n, fill, rows=256, threads=None):
    """Call fill(lo, hi) on row blocks of an n-row matrix from a thread pool
    (NumPy releases the GIL inside its array loops, so the blocks run in
    parallel on the host cores)."""
    blocks = [(lo, min(n, lo + rows)) for lo in range(0, n, rows)]
    with cf.ThreadPoolExecutor(threads or os.cpu_count() or 1) as ex:
        list(ex.map(lambda b: fill(*b), blocks))


def sqdist_rows(x, lo, hi):
    """|x_i - x_j|^2 for rows lo..hi-1 against all points (float64)."""
    D = np.zeros((hi - lo, len(x)))
    for d in range(x.shape[1]):
        D += (x[lo:hi, d, None] - x[None, :, d]) ** 2
    return D


def rbf_kernel(x, s2=1.0, ell=0.2, tau=1e-2):
    x = np.asarray(x, dtype=np.float64)
    n = len(x)
    K = np.empty((n, n))

    def fill(lo, hi):
        K[lo:hi] = s2 * np.exp(-sqdist_rows(x, lo, hi) / (2.0 * ell * ell))

    row_blocks(n, fill)
    K[np.diag_indices(n)] += tau
    return K


def laplacian_2d(m, shift=0.1):
    """CSR of the m*m Dirichlet 5-point Laplacian (4 on the diagonal) + shift I."""
    n = m * m
    main = np.full(n, 4.0 + shift)
    side = -np.ones(n - 1)
    side[np.arange(1, n) % m == 0] = 0.0  # no coupling across grid rows
    updown = -np.ones(n - m)
    A = sp.diags([main, side, side, updown, updown], [0, -1, 1, -m, m], format="csr")
    A.eliminate_zeros()
    A.sort_indices()
    A = sp.csr_matrix((A.data.astype(np.float32), A.indices.astype(np.int32), A.indptr.astype(np.int32)), shape=(n, n))
    return A


def asymmetric_matrix_from_singular_values(vals, nrows, ncols):
    """matfree/test_util.py:33-38: a fixed (nrows, ncols) matrix with singular values vals."""
    A = np.reshape(np.arange(1.0, nrows * ncols + 1.0), (nrows, ncols))
    A /= nrows * ncols
    U, _S, Vt = np.linalg.svd(A, full_matrices=False)
    return U @ np.diag(np.asarray(vals, dtype=np.float64)) @ Vt


def random_csr(n, rng, lengths, band=None):
    """CSR (float64) with lengths[r] entries in row r at distinct random columns,
    within |c - r| <= band when a band is given (sparse-product test matrices)."""
    rows, cols = [], []
    for r in range(n):
        k = int(min(lengths[r], n))
        if band is None:
            cc = rng.choice(n, size=k, replace=False)
        else:
            lo, hi = max(0, r - band), min(n, r + band + 1)
            cc = rng.choice(np.arange(lo, hi), size=min(k, hi - lo), replace=False)
        cols += list(cc)
        rows += [r] * len(cc)
    data = rng.standard_normal(len(rows))
    return sp.csr_matrix((data, (rows, cols)), shape=(n, n))
