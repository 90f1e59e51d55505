"""Philox4x32-10 and the probe samplers, restated in NumPy (oracle; test infrastructure).

Philox4x32 is the counter-based generator of Salmon, Moraes, Dror and Shaw,
"Parallel random numbers: as easy as 1, 2, 3" (SC 2011): ten rounds of two
32x32->64 multiplications with the constants 0xD2511F53 and 0xCD9E8D57, and a
Weyl key schedule with increments 0x9E3779B9 and 0xBB67AE85.  The device
sampler in ``matfree_gb300/csrc`` implements the same mapping; this file
restates it so the Rademacher probes can be checked bit-exactly.

Sample layout (both sides): element (b, i) of a (num, n) probe matrix uses
counter (i // 4, b, stream, 0) and output word i % 4, where stream is 0 for
signs and 1 for normals.  Signs are ``1 - 2 * (word >> 31)``.  Normals use
Box-Muller on the word pairs (0, 1) and (2, 3): u1 = (w0 + 1) 2^-32,
u2 = w1 2^-32, r = sqrt(-2 log u1), z = (r cos 2 pi u2, r sin 2 pi u2).
"""

from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(ctr, key):
    """ctr: uint32 array (..., 4); key: uint32 array (..., 2).  Returns (..., 4)."""
    c = [np.asarray(ctr[..., i], dtype=np.uint32) for i in range(4)]
    k0 = np.asarray(key[..., 0], dtype=np.uint32)
    k1 = np.asarray(key[..., 1], dtype=np.uint32)
    with np.errstate(over="ignore"):
        for r in range(10):
            if r > 0:
                k0 = (k0 + W0).astype(np.uint32)
                k1 = (k1 + W1).astype(np.uint32)
            p0 = M0 * c[0].astype(np.uint64)
            p1 = M1 * c[2].astype(np.uint64)
            hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
            lo0 = (p0 & MASK).astype(np.uint32)
            hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
            lo1 = (p1 & MASK).astype(np.uint32)
            c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
    return np.stack(c, axis=-1)


def prng_key(seed):
    """A key is the 64-bit seed split into two 32-bit words (low, high)."""
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return np.array([seed & 0xFFFFFFFF, seed >> 32], dtype=np.uint32)


def split(key, num=2):
    """Derive ``num`` keys: words 0-1 of philox(ctr=(i, 0, 0, 0x73706c74), key)."""
    i = np.arange(num, dtype=np.uint32)
    ctr = np.stack([i, 0 * i, 0 * i, 0 * i + np.uint32(0x73706C74)], axis=-1)
    out = philox4x32_10(ctr, np.broadcast_to(np.asarray(key, np.uint32), (num, 2)))
    return out[:, :2].copy()


def _words(key, num, n, stream):
    m = (n + 3) // 4
    bi, mi = np.meshgrid(np.arange(num, dtype=np.uint32), np.arange(m, dtype=np.uint32), indexing="ij")
    ctr = np.stack([mi, bi, np.full_like(mi, stream), np.zeros_like(mi)], axis=-1)
    out = philox4x32_10(ctr, np.broadcast_to(np.asarray(key, np.uint32), ctr.shape[:-1] + (2,)))
    return out  # (num, m, 4)


def rademacher(key, num, n):
    """(num, n) float64 array of +-1."""
    w = _words(key, num, n, 0).reshape(num, -1)[:, :n]
    return 1.0 - 2.0 * (w >> np.uint32(31)).astype(np.float64)


def normal(key, num, n):
    """(num, n) float64 standard normals (Box-Muller in float64)."""
    w = _words(key, num, n, 1).astype(np.float64)
    u1a = (w[..., 0] + 1.0) * 2.0**-32
    u2a = w[..., 1] * 2.0**-32
    u1b = (w[..., 2] + 1.0) * 2.0**-32
    u2b = w[..., 3] * 2.0**-32
    ra = np.sqrt(-2.0 * np.log(u1a))
    rb = np.sqrt(-2.0 * np.log(u1b))
    z = np.stack(
        [ra * np.cos(2 * np.pi * u2a), ra * np.sin(2 * np.pi * u2a),
         rb * np.cos(2 * np.pi * u2b), rb * np.sin(2 * np.pi * u2b)], axis=-1)
    return z.reshape(num, -1)[:, :n]
