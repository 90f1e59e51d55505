"""Model of the persistent CTA-pair product's pipeline (CPU only).

`dense_tcgen05_pair_persistent_kernel` runs, per CTA pair, a list of work
items (tile, K range) through four roles that meet only at mbarriers:

* each CTA's producer waits for its ring stage's "empty" phase, the lead CTA
  arms the lead's "full" barrier with both CTAs' bytes, and both CTAs' copies
  complete their bytes on it;
* the lead's MMA thread waits for the accumulator buffer's "tmem_empty" phase
  (items i >= 2 reuse buffer i % 2), then per K slice waits "full", issues the
  MMAs and commits to both CTAs' "empty"; after an item it commits to both
  CTAs' "tmem_full" of the buffer;
* each CTA's four epilogue warps wait "tmem_full", read the accumulator and
  arrive on the lead's "tmem_empty" (8 arrivals complete a phase).

This restates that protocol with the PTX mbarrier semantics (a phase completes
when its pending arrivals and transaction bytes reach zero; a wait on parity
P succeeds once the phase of that parity has completed, so a fresh barrier
passes a wait on parity 1), runs it under many random interleavings with
copies and MMAs completing asynchronously, and checks that every run ends,
that no stage is overwritten while an MMA may read it, that no accumulator
buffer is written by a later item before the epilogue of both CTAs has read
it, and that every epilogue reads a complete accumulator.  The work lists are
the library's own (`mfg_gemm_pair_schedule`).
"""

import ctypes
import random
from collections import defaultdict

import numpy as np
import pytest

from matfree_gb300 import _lib


class Barrier:
    def __init__(self, count):
        self.count = count
        self.pending = count
        self.tx = 0
        self.phase = 0  # completed phases

    def _maybe_complete(self):
        if self.pending == 0 and self.tx == 0:
            self.phase += 1
            self.pending = self.count

    def arrive(self):
        assert self.pending > 0
        self.pending -= 1
        self._maybe_complete()

    def arrive_expect_tx(self, nbytes):
        self.tx += nbytes
        self.arrive()

    def complete_tx(self, nbytes):
        self.tx -= nbytes
        self._maybe_complete()

    def passed(self, parity):
        # the phase with this parity has completed: the current phase's parity differs
        return (self.phase & 1) != parity


def _items(n, p, bn, pairs, min_tail):
    lib = _lib.lib()
    count = lib.mfg_gemm_pair_schedule(n, p, bn, pairs, min_tail, None, 0)
    buf = np.zeros(4 * count, dtype=np.int32)
    lib.mfg_gemm_pair_schedule(n, p, bn, pairs, min_tail, ctypes.c_void_p(buf.ctypes.data), count)
    per_pair = defaultdict(list)
    for q, t, kb, ke in buf.reshape(count, 4):
        per_pair[int(q)].append((int(t), int(kb), int(ke)))
    return per_pair


def simulate(items, stages, rng, stage_bytes=64, empty_parity=lambda use: (use - 1) & 1):
    """One pair: returns the number of scheduler steps (asserts on any violation)."""
    full = [Barrier(1) for _ in range(stages)]                      # the lead's
    empty = [[Barrier(1) for _ in range(stages)] for _ in range(2)]  # per CTA
    tfull = [[Barrier(1) for _ in range(2)] for _ in range(2)]       # per CTA, per buffer
    tempty = [Barrier(8) for _ in range(2)]                          # the lead's
    slices = [(i, kt) for i, (_, kb, ke) in enumerate(items) for kt in range(kb, ke)]
    stage_owner = [None] * stages        # global slice index whose data the stage holds
    stage_readers = [0] * stages         # MMAs issued on the stage and not complete
    acc_item = [None, None]              # item whose MMAs write the buffer
    acc_done = defaultdict(int)          # completed MMA slices per item
    acc_issued = defaultdict(int)
    acc_read = defaultdict(int)          # epilogue warps (of 8) that read the item
    events = []                          # asynchronous completions: (kind, payload)

    def producer(cta):
        for g, _ in enumerate(slices):
            s, ph = g % stages, (g // stages) & 1
            while not empty[cta][s].passed(ph ^ 1):
                yield
            if cta == 0:
                full[s].arrive_expect_tx(2 * stage_bytes)
                # the stage is being refilled: every MMA that read it has completed
                assert stage_readers[s] == 0
                stage_owner[s] = g
            events.append(("copy", (s, g)))
            yield

    def mma():
        g = 0
        for i, (_, kb, ke) in enumerate(items):
            buf, use = i & 1, i >> 1
            if use > 0:
                while not tempty[buf].passed(empty_parity(use)):
                    yield
                # both CTAs' epilogues have read the buffer's previous item
                assert acc_read[i - 2] == 8
            acc_item[buf] = i
            for _ in range(kb, ke):
                s, ph = g % stages, (g // stages) & 1
                while not full[s].passed(ph):
                    yield
                assert stage_owner[s] == g
                stage_readers[s] += 1
                acc_issued[i] += 1
                events.append(("mma", (s, i)))
                events.append(("commit_empty", (s, acc_issued[i], i)))
                g += 1
                yield
            events.append(("commit_tfull", (buf, i, ke - kb)))
            yield

    def epilogue(cta, warp):
        for i, (_, kb, ke) in enumerate(items):
            buf, use = i & 1, i >> 1
            while not tfull[cta][buf].passed(use & 1):
                yield
            # a complete accumulator of this item, not yet overwritten
            assert acc_done[i] == ke - kb and acc_item[buf] == i
            acc_read[i] += 1
            yield
            tempty[buf].arrive()
            yield

    actors = [producer(0), producer(1), mma()] + [epilogue(c, w) for c in range(2) for w in range(4)]
    alive = list(actors)
    steps = 0
    while alive or events:
        steps += 1
        assert steps < 200000, "no progress: the protocol deadlocks"
        # an asynchronous completion or a role step, at random
        if events and (not alive or rng.random() < 0.4):
            # commits complete in order after the MMAs before them; copies land in any order
            kinds = [k for k, _ in events]
            j = rng.randrange(len(events))
            kind, payload = events[j]
            if kind in ("commit_empty", "commit_tfull", "mma"):
                j = kinds.index(next(k for k in kinds if k in ("commit_empty", "commit_tfull", "mma")))
                kind, payload = events[j]
            events.pop(j)
            if kind == "copy":
                s, g = payload
                full[s].complete_tx(stage_bytes)
            elif kind == "mma":
                s, i = payload
                stage_readers[s] -= 1
                acc_done[i] += 1
            elif kind == "commit_empty":
                s, _, _ = payload
                for c in range(2):
                    empty[c][s].arrive()
            else:
                buf, i, nsl = payload
                assert acc_done[i] == nsl
                for c in range(2):
                    tfull[c][buf].arrive()
            continue
        a = rng.choice(alive)
        try:
            next(a)
        except StopIteration:
            alive.remove(a)
    assert all(acc_read[i] == 8 for i in range(len(items)))
    return steps


@pytest.mark.parametrize("n,p,bn,pairs", [(16384, 256, 256, 76), (11584, 256, 256, 76),
                                          (5000, 700, 256, 76), (4608, 256, 256, 76),
                                          (20000, 64, 64, 76), (3000, 256, 128, 7)])
def test_persistent_pipeline_protocol(n, p, bn, pairs):
    stages = 6
    per_pair = _items(n, p, bn, pairs, stages)
    rng = random.Random(n * 7 + p)
    # the pairs with the most items exercise buffer reuse; K ranges scaled down
    # to keep the model quick (the protocol does not depend on their length)
    chosen = sorted(per_pair, key=lambda q: -len(per_pair[q]))[:3]
    for q in chosen:
        items = [(t, 0, min(ke - kb, 9)) for t, kb, ke in per_pair[q]]
        for _ in range(20):
            simulate(items, stages, rng)


def test_model_catches_a_missing_release():
    # the model itself: an epilogue that never releases the accumulator must deadlock
    items = [(0, 0, 3), (1, 0, 3), (2, 0, 3)]
    rng = random.Random(0)
    original = Barrier.arrive

    def drop_tempty(self):
        if self.count == 8:
            return  # release lost
        original(self)

    Barrier.arrive = drop_tempty
    try:
        with pytest.raises(AssertionError, match="deadlocks"):
            simulate(items, 4, rng)
    finally:
        Barrier.arrive = original


def test_model_catches_a_wrong_release_parity():
    # waiting on the parity of the current use instead of the previous one lets
    # the MMAs overwrite an accumulator the epilogues have not read
    items = [(t, 0, 4) for t in range(6)]
    caught = 0
    for seed in range(20):
        try:
            simulate(items, 4, random.Random(seed), empty_parity=lambda use: use & 1)
        except AssertionError:
            caught += 1
    assert caught > 0
