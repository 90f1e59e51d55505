"""Monte-Carlo estimators and probe samplers (GPU).

``estimator_monte_carlo(integrand, /, sampler)`` and
``estimator_monte_carlo_mean_and_sem`` follow matfree/stochtrace.py:7-89:
``estimate(matvec, key, *params)`` draws the probes, evaluates the integrand
on every probe and averages.  matfree vmaps the integrand; here SLQ
integrands evaluate all probes in one batched library call, and other
integrands are evaluated probe by probe on the GPU.

``sampler_signs`` / ``sampler_normal`` (stochtrace.py:927-977) draw their
probes on the device with Philox4x32-10; ``sampler_rademacher`` is the
spec name of ``sampler_signs``.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._panel import dtype_code, empty_panel, require_cuda, stream_ptr
from .tree import ravel_pytree, tree_map


class _Sampler:
    def __init__(self, kind, args_like, num):
        flat, unravel = ravel_pytree(args_like[0] if len(args_like) == 1 else args_like)
        flat = require_cuda(flat, "args_like")
        if flat.dtype.is_complex:
            raise NotImplementedError("complex probes (Steinhaus) are not provided by matfree_gb300")
        self.kind = kind
        self.n = flat.numel()
        self.dtype = flat.dtype if flat.dtype in (torch.float32, torch.float64) else torch.float32
        self.device = flat.device
        self.num = int(num)
        self.unravel = unravel
        self.is_flat = flat.dim() == 1 and not isinstance(args_like[0], (dict, list, tuple))

    def panel(self, key) -> torch.Tensor:
        """The (num, n) probe matrix as a view of a padded device panel."""
        key = np.ascontiguousarray(np.asarray(key, dtype=np.uint32).reshape(2))
        out = empty_panel(self.num, self.n, self.dtype, self.device)
        fn = _lib.lib().mfg_sampler_signs if self.kind == "signs" else _lib.lib().mfg_sampler_normal
        st = fn(key.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), self.num, self.n, out.shape[1],
                dtype_code(self.dtype), ctypes.c_void_p(out.data_ptr()), stream_ptr())
        _lib.check(st, "sampler")
        return out[:, : self.n]

    def __call__(self, key):
        flat = self.panel(key)
        if self.is_flat:
            return flat
        return _Samples(flat, self.unravel)


class _Samples:
    """Pytree-valued samples that keep the flat device panel for batched use."""

    def __init__(self, flat, unravel):
        self.flat = flat
        self.unravel = unravel  # one flat row -> one pytree sample
        self.tree = unravel(flat)


def sampler_signs(*args_like, num):
    """Rademacher +-1 probes (matfree/stochtrace.py:932-937)."""
    return _Sampler("signs", args_like, num)


sampler_rademacher = sampler_signs


def sampler_normal(*args_like, num):
    """Standard-normal probes (matfree/stochtrace.py:927-929)."""
    return _Sampler("normal", args_like, num)


def _evaluate(integrand, matvec, samples, parameters):
    flat = samples.flat if isinstance(samples, _Samples) else samples
    if hasattr(integrand, "batched") and isinstance(flat, torch.Tensor) and flat.dim() == 2:
        if isinstance(samples, _Samples) and not hasattr(matvec, "c_struct"):
            # pytree probes with a pytree matvec: flatten the matvec
            unravel = samples.unravel

            def flat_matvec(v, *p):
                return ravel_pytree(matvec(_unbatch(unravel, v), *p))[0]

            return integrand.batched(flat_matvec, flat, *parameters)
        return integrand.batched(matvec, flat, *parameters)
    rows = samples.tree if isinstance(samples, _Samples) else samples
    leaves = [integrand(matvec, _index(rows, i), *parameters) for i in range(flat.shape[0])]
    return tree_map(lambda *xs: torch.stack(xs), *leaves)


def _unbatch(unravel, v):
    return unravel(v)


def _index(tree, i):
    if isinstance(tree, torch.Tensor):
        return tree[i]
    return tree_map(lambda x: x[i], tree)


def estimator_monte_carlo(integrand, /, sampler):
    """matfree/stochtrace.py:7-52."""

    def estimate(matvecs, key, *parameters):
        samples = sampler(key)
        Qs = _evaluate(integrand, matvecs, samples, parameters)
        return tree_map(lambda s: torch.mean(s, dim=0), Qs)

    return estimate


def estimator_monte_carlo_mean_and_sem(integrand, /, sampler):
    """matfree/stochtrace.py:55-89: (mean, std / sqrt(num))."""

    def estimate(matvecs, key, *parameters):
        samples = sampler(key)
        Qs = _evaluate(integrand, matvecs, samples, parameters)
        mean = tree_map(lambda s: torch.mean(s, dim=0), Qs)
        sem = tree_map(lambda s: torch.std(s, dim=0, correction=0) / np.sqrt(s.shape[0]), Qs)
        return mean, sem

    return estimate
