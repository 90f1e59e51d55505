"""CPU oracle for the SLQ log-determinant path (test infrastructure only).

This package restates, in float64 NumPy, the algorithm that matfree runs on the
stochastic-Lanczos-quadrature path.  It is the checker for the CUDA library in
``matfree_gb300``: tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` may call it; the product path never does.

Parity status: matfree is pure JAX and JAX cannot be imported where this oracle
was written, so the reference itself cannot be executed.  The oracle is pinned
instead against every known-answer test that matfree's own test-suite holds for
this path (``tests/test_oracle_kats.py`` ports them):

* full-rank reconstruction ``Q^T T Q = A`` (tests/test_decomp/test_tridiag_sym.py:7-38)
* Arnoldi/Lanczos relation ``A Q^T - Q^T T - r e_k^T = 0`` (test_tridiag_sym.py:43-65,
  test_hessenberg.py:7-69, including the Hilbert-matrix case)
* output shapes and the ``exceeds`` error (test_consistency.py:26-63)
* SLQ log-det vs ``slogdet`` (test_monte_carlo_funm_sym_logdet.py:16-38)
* ``v^T log(A) v`` exactness at k = n - 1 (test_monte_carlo_funm_sym_logdet.py:41-67)
* the Hessenberg adjoint against differentiation of the forward pass
  (test_hessenberg_adjoint.py, test_tridiag_sym_adjoint.py; finite differences
  stand in for JAX autodiff)

Random probes: matfree draws them with ``jax.random`` (threefry).  Bit-parity
with ``jax.random`` is unpinned; parity tests pass explicit probe matrices to
both sides, and ``oracle.philox`` restates this library's own counter-based
generator so that the device sampler is checked bit-exactly.
"""
