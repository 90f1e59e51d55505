"""CPU transliteration of the CSR SpMM kernel's index arithmetic
(csr_spmm_window_kernel in matfree_gb300/csrc/operators.cu): tiles of rows,
the first RMAX entries of each row in registers (padding: the row's own
column with a zero value) and the rest from global memory, the window [lo,
lo + wlen) of each probe vector that a tile reads (bounds: inside the padded
panel row, every gather inside the window), the windowed path, the per-lane
gather path and the warp-cooperative long-row path, checked against scipy on
stencils, ragged and empty rows, rows longer than the registers and than a
warp, and windows wider than a ring buffer."""

import numpy as np
import pytest
import scipy.sparse as sp

from oracle.problems import random_csr as _random_csr

ROWS, THREADS, WMAX, LONG = 1024, 256, 4096, 32


def spmm_model(rp, ci, val, n, V, ld, shift, rmax=6, tr=ROWS):
    p = V.shape[0]
    W = np.full((p, n), np.nan)
    paths = set()
    assert 1 <= tr <= ROWS
    for tile in range((n + tr - 1) // tr):
        r0 = tile * tr
        rows = min(tr, n - r0)
        s_rp = rp[r0:r0 + rows + 1]
        lo_, hi_ = r0, r0 + rows - 1
        # per row thread: the first rmax entries in registers (padded with the
        # row's own column and a zero value), the rest read from global memory
        regs = {}
        for lr in range(rows):
            e0, e1 = int(s_rp[lr]), int(s_rp[lr + 1])
            cols = [int(ci[e]) if e < e1 else r0 + lr for e in range(e0, e0 + rmax)]
            vals = [val[e] if e < e1 else 0.0 for e in range(e0, e0 + rmax)]
            regs[lr] = (cols, vals, e0, e1)
            for e in range(e0, e1):
                lo_, hi_ = min(lo_, int(ci[e])), max(hi_, int(ci[e]))
        lo = lo_ & ~3
        wlen = (hi_ + 1 - lo + 3) & ~3
        windowed = wlen <= WMAX and lo_ >= 0 and hi_ < n
        if windowed:
            assert lo % 4 == 0 and lo + wlen <= ld
            paths.add("window")
            for b in range(p):
                win = V[b, lo:lo + wlen]  # one bulk copy of wlen * 4 bytes
                for lr in range(rows):
                    cols, vals, e0, e1 = regs[lr]
                    acc = np.float32(shift) * np.float32(win[r0 + lr - lo])
                    for c, a in zip(cols, vals):
                        assert 0 <= c - lo < wlen
                        acc = np.float32(acc + np.float32(a) * np.float32(win[c - lo]))
                    for e in range(e0 + rmax, e1):
                        assert 0 <= ci[e] - lo < wlen
                        acc = np.float32(acc + np.float32(val[e]) * np.float32(win[ci[e] - lo]))
                    W[b, r0 + lr] = acc
            continue
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
                                assert 0 <= ci[e] < n
                                acc = np.float32(acc + np.float32(val[e]) * np.float32(V[b, ci[e]]))
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
                                    assert 0 <= ci[e] < n
                                    parts[ln] += val[e] * V[b, ci[e]]
                            W[b, r0 + lj] = shift * V[b, r0 + lj] + parts.sum()
    return W, paths


@pytest.mark.parametrize("case,paths", [("stencil", {"window"}), ("banded_ragged", {"window"}),
                                        ("random_ragged", {"gather"}), ("long", {"gather", "long"}),
                                        ("wide_rows", {"window"}), ("empty_tail", {"window"})])
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
        n = 9000
        lens = rng.integers(1, 4, size=n)
        lens[[5, 1130, 4100]] = [70, 200, 33]
        A = _random_csr(n, rng, lens)
    elif case == "wide_rows":
        n = 1100
        A = _random_csr(n, rng, np.full(n, 40))  # 40 entries per row: most beyond the registers
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
    for rmax in (6, 12):
        got, seen = spmm_model(rp, ci, val, n, V, ld, 0.3, rmax)
        assert seen == paths
        np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-5)
