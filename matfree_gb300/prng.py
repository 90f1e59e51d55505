"""Keys for the counter-based probe generator (Philox4x32-10).

Mirrors matfree/backend/prng.py:6-11 (``prng_key``, ``split``) in spirit: a
key is a pair of 32-bit words; samples are a pure function of (key, shape),
generated on the GPU by the samplers in ``stochtrace``.  Philox4x32-10 is the
generator of Salmon et al. (SC 2011); ``split`` runs it here on the host.
Bit-compatibility with ``jax.random`` (threefry) is not provided.
"""

from __future__ import annotations

import numpy as np

_M0, _M1 = 0xD2511F53, 0xCD9E8D57
_W0, _W1 = 0x9E3779B9, 0xBB67AE85
_SPLIT_TAG = 0x73706C74


def _philox(ctr, key):
    c0, c1, c2, c3 = (int(x) & 0xFFFFFFFF for x in ctr)
    k0, k1 = (int(x) & 0xFFFFFFFF for x in key)
    for r in range(10):
        if r:
            k0 = (k0 + _W0) & 0xFFFFFFFF
            k1 = (k1 + _W1) & 0xFFFFFFFF
        p0 = _M0 * c0
        p1 = _M1 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF, ((p0 >> 32) ^ c3 ^ k1) & 0xFFFFFFFF, p0 & 0xFFFFFFFF
    return c0, c1, c2, c3


def prng_key(seed: int) -> np.ndarray:
    """A key from an integer seed: the low and high 32-bit words."""
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return np.array([seed & 0xFFFFFFFF, seed >> 32], dtype=np.uint32)


PRNGKey = prng_key


def split(key, num: int = 2) -> np.ndarray:
    """``num`` new keys: words 0-1 of philox((i, 0, 0, tag), key)."""
    key = np.asarray(key, dtype=np.uint32).reshape(2)
    out = np.zeros((num, 2), dtype=np.uint32)
    for i in range(num):
        w = _philox((i, 0, 0, _SPLIT_TAG), key)
        out[i] = w[:2]
    return out
