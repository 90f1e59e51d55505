"""Geometry of the two-sweep passes over at most 8 vectors (CPU only).

These passes of `stream_sweep_kernel` take chunks of 512 rows (kRPT = 4 rows a
row thread, 128 row threads) and load every vector of a chunk with one 1-D
bulk copy.  This restates the kernel's arithmetic (the flat chunk walk b * C +
c cut into equal CTA ranges, r0 = c * 512, rows = min(n - r0, 512), a copy of
round_up(4 * rows, 16) bytes per vector into a [cpad + 2][512] buffer, thread
j owning rows j + 128 rr) and checks for many n, p, vector counts and grids:

* every row of every probe is handled by exactly one (CTA, chunk, thread, rr);
* the buffer indices of the row threads stay inside their buffer;
* the copies' bytes sum to the bytes the "full" barrier expects;
* no copy reads past a vector's padded row (ld = round_up(n, 8) floats), and
  no store goes past n.
"""

import pytest

KSR, KRPT, KSPG, NV = 128, 4, 8, 2
CR = KSR * KRPT


def _ld(n):
    return (n + 7) // 8 * 8


def _thread_rows():
    """Rows of a chunk each (thread, rr) owns: every row 0 .. CR - 1 exactly once."""
    rows = sorted(j + rr * KSR for j in range(KSR) for rr in range(KRPT))
    assert rows == list(range(CR))
    return rows


def _check(n, p, ncols, G):
    C = -(-n // CR)
    F = p * C
    cpad = -(-ncols // KSPG) * KSPG
    bstr = (cpad + NV) * CR
    # every buffer read of a row thread (vectors 0 .. cpad + 1 at its row < CR)
    assert (cpad + NV - 1) * CR + (CR - 1) < bstr
    covered = {}
    for x in range(G):
        f0, f1 = F * x // G, F * (x + 1) // G
        for f in range(f0, f1):
            b, c = divmod(f, C)
            r0 = c * CR
            rows = min(n - r0, CR)
            assert rows > 0
            seg = -(-rows * 4 // 16) * 16
            assert seg <= CR * 4  # a copy fits its slot of the buffer
            # every copy reads r0 .. r0 + seg / 4 of one vector: inside the padded row
            assert r0 + seg // 4 <= _ld(n)
            # expect_tx: one 1-D copy of seg bytes per vector, no 2-D copies
            assert seg * (ncols + NV) == sum([seg] * (ncols + NV))
            # rows jr < rows of the chunk are handled (and stored: r0 + jr < n)
            covered.setdefault(b, []).append((r0, r0 + rows))
    assert sorted(covered) == list(range(p))
    for b, iv in covered.items():
        iv.sort()
        assert iv[0][0] == 0 and iv[-1][1] == n
        assert all(a[1] == c[0] for a, c in zip(iv, iv[1:])), (b, iv)


@pytest.mark.parametrize("n", [512, 513, 1000, 1024, 4099, 11992, 16384, 21717, 29867])
@pytest.mark.parametrize("p", [1, 32, 64, 256])
@pytest.mark.parametrize("ncols", [1, 5, 8])
def test_sweep_chunk_geometry(n, p, ncols):
    _thread_rows()
    C = -(-n // CR)
    for G in sorted({1, min(304, p * C), max(1, p * C // 3)}):
        _check(n, p, ncols, G)
