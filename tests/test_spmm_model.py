"""CPU transliteration of the CSR SpMM kernel's index arithmetic
(csr_spmm_window_kernel in matfree_gb300/csrc/operators.cu): tiles of rows,
the staging of a tile's CSR segment in 4-entry chunks, the window [lo, lo +
wlen) of each probe vector that a tile reads (bounds: inside the padded
panel row, every gather inside the window), the windowed path, the
per-lane gather path and the warp-cooperative long-row path, checked
against scipy on stencils, ragged and empty rows, unaligned segment starts,
rows longer than a warp, segments longer than the staging buffer and
windows wider than a ring buffer."""

import numpy as np
import pytest
import scipy.sparse as sp

from oracle.problems import random_csr as _random_csr

ROWS, THREADS, SEG, WMAX, LONG = 1024, 256, 6144, 4096, 32


def spmm_model(rp, ci, val, n, V, ld, shift, vec_ok=True):
    nnz = len(ci)
    p = V.shape[0]
    W = np.full((p, n), np.nan)
    paths = set()
    for tile in range((n + ROWS - 1) // ROWS):
        r0 = tile * ROWS
        rows = min(ROWS, n - r0)
        s_rp = rp[r0:r0 + rows + 1]
        e_begin, e_end = int(s_rp[0]), int(s_rp[rows])
        a0 = e_begin & ~3
        staged = e_end - a0 <= SEG
        lo_, hi_ = r0, r0 + rows - 1
        s_ci = np.full(SEG + 8, -1, dtype=np.int64)
        s_val = np.full(SEG + 8, np.nan)
        if staged:
            for q in range((e_end - a0 + 3) >> 2):
                e = a0 + 4 * q
                for t in range(4):
                    if vec_ok and e + 4 <= nnz:
                        assert e % 4 == 0
                    s_ci[4 * q + t] = ci[e + t] if e + t < nnz else 0
                    s_val[4 * q + t] = val[e + t] if e + t < nnz else 0.0
                    if e_begin <= e + t < e_end:
                        lo_, hi_ = min(lo_, s_ci[4 * q + t]), max(hi_, s_ci[4 * q + t])
        lo = lo_ & ~3
        wlen = (hi_ + 1 - lo + 3) & ~3
        assert lo >= 0 and lo % 4 == 0 and lo + wlen <= ld
        windowed = staged and wlen <= WMAX
        if windowed:
            paths.add("window")
            for b in range(p):
                win = V[b, lo:lo + wlen]  # one bulk copy of wlen * 4 bytes
                for t in range(THREADS):
                    for i in range(ROWS // THREADS):
                        lr = t + i * THREADS
                        if lr >= rows:
                            continue
                        acc = np.float32(shift) * np.float32(win[r0 + lr - lo])
                        for e in range(int(s_rp[lr]), int(s_rp[lr + 1])):
                            k = s_ci[e - a0] - lo
                            assert 0 <= k < wlen
                            acc = np.float32(acc + np.float32(s_val[e - a0]) * np.float32(win[k]))
                        W[b, r0 + lr] = acc
            continue

        def col_at(e):
            return s_ci[e - a0] if staged else ci[e]

        def val_at(e):
            return s_val[e - a0] if staged else val[e]

        for i in range(ROWS // THREADS):
            for warp in range(THREADS // 32):
                lrs = [warp * 32 + lane + i * THREADS for lane in range(32)]
                lens = [int(s_rp[lr + 1] - s_rp[lr]) if lr < rows else 0 for lr in lrs]
                if max(lens) <= LONG:
                    paths.add("gather")
                    for lr in lrs:
                        if lr >= rows:
                            continue
                        for b in range(p):
                            acc = np.float32(shift) * np.float32(V[b, r0 + lr])
                            for e in range(int(s_rp[lr]), int(s_rp[lr + 1])):
                                c = col_at(e)
                                assert 0 <= c < n
                                acc = np.float32(acc + np.float32(val_at(e)) * np.float32(V[b, c]))
                            W[b, r0 + lr] = acc
                else:
                    paths.add("long")
                    for j in range(32):
                        lj = lrs[0] + j
                        if lj >= rows:
                            break
                        f0, f1 = int(s_rp[lj]), int(s_rp[lj + 1])
                        for b in range(p):
                            parts = np.zeros(32)
                            for ln in range(32):
                                for e in range(f0 + ln, f1, 32):
                                    c = col_at(e)
                                    assert 0 <= c < n
                                    parts[ln] += val_at(e) * V[b, c]
                            W[b, r0 + lj] = shift * V[b, r0 + lj] + parts.sum()
    return W, paths


@pytest.mark.parametrize("case,paths", [("stencil", {"window"}), ("banded_ragged", {"window"}),
                                        ("random_ragged", {"gather"}), ("long", {"gather", "long"}),
                                        ("huge_segment", {"long", "window"}), ("empty_tail", {"window"})])
def test_spmm_model_matches_scipy(case, paths):
    rng = np.random.default_rng(len(case))
    if case == "stencil":
        m = 45
        n = m * m
        A = sp.diags([4.0, -1.0, -1.0, -1.0, -1.0], [0, -1, 1, -m, m], shape=(n, n), format="csr")
    elif case == "banded_ragged":
        n = 2500
        A = _random_csr(n, rng, rng.integers(0, 9, size=n), band=700)
    elif case == "random_ragged":
        n = 6000
        A = _random_csr(n, rng, rng.integers(0, 4, size=n))
    elif case == "long":
        n = 5000
        lens = rng.integers(1, 4, size=n)
        lens[[5, 1130, 4100]] = [70, 200, 33]
        A = _random_csr(n, rng, lens)
    elif case == "huge_segment":
        n = 1100
        A = _random_csr(n, rng, np.full(n, 40))  # 1024 rows x 40 > 6144 staged entries
    else:
        n = 1500
        lens = rng.integers(0, 4, size=n)
        lens[-600:] = 0
        A = _random_csr(n, rng, lens, band=300)
    A.sort_indices()
    rp = A.indptr.astype(np.int64)
    ci = A.indices.astype(np.int64)
    val = A.data.astype(np.float32).astype(np.float64)
    ld = (n + 7) // 8 * 8
    V = np.zeros((3, ld))
    V[:, :n] = rng.standard_normal((3, n)).astype(np.float32)
    want = (A.astype(np.float64) @ V[:, :n].T).T + 0.3 * V[:, :n]
    for vec_ok in (True, False):
        got, seen = spmm_model(rp, ci, val, n, V, ld, 0.3, vec_ok)
        assert seen == paths
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-5)
