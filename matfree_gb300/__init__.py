"""matfree_gb300: stochastic Lanczos quadrature on GB300 (sm_103a).

A drop-in for the SLQ log-determinant path of pnkraemer/matfree:
``stochtrace.estimator_monte_carlo(funm.monte_carlo_funm_sym_logdet(
decomp.tridiag_sym(k)), stochtrace.sampler_signs(x_like, num=p))`` with the
operator applied to all probes at once by CUDA kernels in
``libmatfree_gb300.so`` (C ABI: include/matfree_gb300.h).
"""

from . import decomp, funm, gp, linalg, operators, prng, stochtrace, tree  # noqa: F401
from ._lib import library_path, lib  # noqa: F401
from .operators import CallbackOperator, CSROperator, DenseOperator, RBFKernelOperator  # noqa: F401

__all__ = [
    "decomp", "funm", "stochtrace", "prng", "operators", "tree", "linalg", "gp",
    "DenseOperator", "RBFKernelOperator", "CSROperator", "CallbackOperator",
    "lib", "library_path",
]
