"""Schedule of the persistent CTA-pair operator product (CPU only).

The library's own schedule code (``mfg_gemm_pair_schedule``: the same
``pair_schedule`` / ``pair_item`` functions the kernel runs) is enumerated
for many operator sizes, probe counts and SM counts, and checked for what the
kernel's correctness rests on:

* every (tile, K slice) of the product is computed exactly once;
* a tile is either whole or split into exactly two pieces, one starting at
  K slice 0 (it adds the shift term), so the two partial products add into a
  zeroed output in an order that cannot change the sum;
* every item lies inside the grid (pair < P, tile < T, 0 <= kb < ke <= K);
* if any tile is split, every tile is split at the same K slice: the tensor
  pipe's accumulation rounding depends on the chain length, and a mix of
  split and unsplit rows would make a symmetric operator non-symmetric;
* the busiest pair's K slices match the schedule's cost (n = 16384, 256
  probes on 76 pairs: 439 of 512).
"""

import ctypes
from collections import defaultdict

import numpy as np
import pytest

from matfree_gb300 import _lib


def _items(n, p, bn, pairs, min_tail):
    lib = _lib.lib()
    count = lib.mfg_gemm_pair_schedule(n, p, bn, pairs, min_tail, None, 0)
    assert count > 0, count
    buf = np.zeros(4 * count, dtype=np.int32)
    got = lib.mfg_gemm_pair_schedule(n, p, bn, pairs, min_tail, ctypes.c_void_p(buf.ctypes.data), count)
    assert got == count
    return buf.reshape(count, 4)


def _check(n, p, bn, pairs, min_tail):
    K = -(-n // 32)
    tiles_m = -(-n // 256)
    T = tiles_m * -(-p // bn)
    items = _items(n, p, bn, pairs, min_tail)
    assert np.all(items[:, 0] >= 0) and np.all(items[:, 0] < pairs)
    assert np.all(items[:, 1] >= 0) and np.all(items[:, 1] < T)
    assert np.all(items[:, 2] >= 0) and np.all(items[:, 2] < items[:, 3]) and np.all(items[:, 3] <= K)
    pieces = defaultdict(list)
    for _, t, kb, ke in items:
        pieces[int(t)].append((int(kb), int(ke)))
    assert sorted(pieces) == list(range(T))
    for t, ps in pieces.items():
        ps.sort()
        assert len(ps) in (1, 2), (t, ps)
        assert ps[0][0] == 0 and ps[-1][1] == K, (t, ps)
        if len(ps) == 2:
            assert ps[0][1] == ps[1][0], (t, ps)
            assert ps[1][1] - ps[1][0] >= min_tail
    splits = {ps[0][1] for ps in pieces.values() if len(ps) == 2}
    if splits:
        assert len(splits) == 1 and all(len(ps) == 2 for ps in pieces.values()), splits
    load = defaultdict(int)
    for q, _, kb, ke in items:
        load[int(q)] += int(ke - kb)
    return max(load.values()), K, T


def test_headline_shape_spreads_the_last_wave():
    busiest, K, T = _check(16384, 256, 256, 76, 6)
    assert (K, T) == (512, 64)
    assert busiest == 439  # against 512 with one tile per pair
    items = _items(16384, 256, 256, 76, 6)
    assert len(set(items[:, 0])) == 76  # every pair works


@pytest.mark.parametrize("n", [1024, 1448, 2048, 4096, 5000, 8192, 11584, 16384, 20000, 23168, 32768, 40000])
@pytest.mark.parametrize("p,bn", [(32, 32), (100, 112), (128, 128), (256, 256), (256, 128), (512, 256), (700, 256)])
@pytest.mark.parametrize("pairs", [76, 74, 7])
def test_every_slice_once_and_at_most_two_pieces(n, p, bn, pairs):
    busiest, K, T = _check(n, p, bn, pairs, 6)
    waves = -(-T // pairs)
    assert busiest <= waves * K


def test_bad_arguments():
    lib = _lib.lib()
    assert lib.mfg_gemm_pair_schedule(0, 256, 256, 76, 6, None, 0) < 0
    assert lib.mfg_gemm_pair_schedule(1024, 256, 200, 76, 6, None, 0) < 0
    assert lib.mfg_gemm_pair_schedule(1024, 256, 256, 1, 6, None, 0) < 0
