"""The continuous-batching server: alone == in the mix, admission, parity."""

import numpy as np
import pytest

from matfree_gb300 import serve
from oracle import philox, problems, slq

pytestmark = pytest.mark.gpu

# a solve that does not finish fails the test instead of blocking the suite
STALL_S = 120.0


def _requests(num=6, seed=3):
    reqs = serve.synthetic_stream(num, rate=1e6, seed=seed, n_range=(512, 2048), ks=(16, 24),
                                  ps=(32, 64))
    for r in reqs:
        r.arrival = 0.0
    return reqs


def test_result_is_identical_alone_and_in_the_mix():
    # without packing: every request is its own solve, on its own stream
    reqs = _requests()
    alone = []
    for r in reqs:
        res, _ = serve.SLQServer(slots=1, group_max_n=0).run([r], realtime=False, stall_s=STALL_S)
        alone.append(res[0])
    mixed, stats = serve.SLQServer(slots=4, group_max_n=0).run(reqs, realtime=False, stall_s=STALL_S)
    assert stats["solves"] == len(reqs) and stats["packed_solves"] == 0
    for a, m in zip(alone, mixed):
        assert a.rid == m.rid
        assert a.mean == m.mean and a.sem == m.sem  # bit-identical: deterministic kernels


def test_packed_requests_match_their_alone_values():
    # small requests of the same k and f share one solve (zero-padded to a
    # common n, block-diagonal operator); each value equals its alone value up
    # to the order of floating-point sums
    reqs = serve.synthetic_stream(12, rate=1e6, seed=5, n_range=(600, 1100), ks=(24,), ps=(32, 64),
                                  funs=("log",))
    for r in reqs:
        r.arrival = 0.0
    alone = {}
    for r in reqs:
        res, _ = serve.SLQServer(slots=1, group_max_n=0).run([r], realtime=False, stall_s=STALL_S)
        alone[r.rid] = res[0]
    packed, stats = serve.SLQServer(slots=2).run(reqs, realtime=False, stall_s=STALL_S)
    assert stats["solves"] == len(reqs)
    assert stats["packed_solves"] >= 1 and stats["packed_requests"] >= 4
    for m in packed:
        a = alone[m.rid]
        assert abs(m.mean - a.mean) <= 1e-5 * abs(a.mean), (m.rid, m.mean, a.mean)
        assert abs(m.sem - a.sem) <= 1e-3 * abs(a.sem)


@pytest.mark.parametrize("fun", ["log", "exp:-0.1"])
def test_packed_group_matches_oracle(fun):
    reqs = serve.synthetic_stream(5, rate=1e6, seed=8, n_range=(700, 1300), ks=(20,), ps=(32,),
                                  funs=(fun,))
    for r in reqs:
        r.arrival = 0.0
    res, stats = serve.SLQServer(slots=1).run(reqs, realtime=False, stall_s=STALL_S)
    assert stats["packed_requests"] == len(reqs)
    f = np.log if fun == "log" else (lambda t: np.exp(-0.1 * t))
    for r, got in zip(reqs, res):
        n = r.x.shape[0]
        K = problems.rbf_kernel(r.x.astype(np.float64))
        V = philox.rademacher(np.asarray(r.key, dtype=np.uint32), r.p, n)
        want = slq.slq_batched(lambda X: X @ K, r.k, V, matfun=f)
        assert got.rid == r.rid
        assert abs(got.mean - want.mean()) <= 1e-4 * abs(want.mean()), (r.rid, n)


def test_admission_respects_the_memory_budget():
    reqs = _requests(num=5, seed=4)
    biggest = max(serve.footprint_bytes(r.x.shape[0], r.k, r.p, "bf16x3") for r in reqs)
    server = serve.SLQServer(slots=4, budget_bytes=1.5 * biggest, group_max_n=0)
    seen = []
    orig = server._launch

    def spy(slot, req):
        seen.append(server.used)
        return orig(slot, req)

    server._launch = spy
    res, stats = server.run(reqs, realtime=False, stall_s=STALL_S)
    assert stats["solves"] == len(reqs)
    assert max(seen) <= 1.5 * biggest
    with pytest.raises(ValueError, match="budget"):
        serve.SLQServer(slots=1, budget_bytes=biggest / 10, group_max_n=0).run(reqs[:1], realtime=False, stall_s=STALL_S)


@pytest.mark.parametrize("fun", ["log", "exp:-0.1"])
def test_served_value_matches_oracle(fun):
    n, k, p = 1024, 24, 32
    x = problems.rbf_points(n, seed=9).astype(np.float32)
    req = serve.Request(rid=0, x=x, k=k, p=p, fun=fun, key=(7, 0))
    (res,), _ = serve.SLQServer(slots=1).run([req], realtime=False, stall_s=STALL_S)
    K = problems.rbf_kernel(x.astype(np.float64))
    V = philox.rademacher(np.array([7, 0], dtype=np.uint32), p, n)
    f = np.log if fun == "log" else (lambda t: np.exp(-0.1 * t))
    want = slq.slq_batched(lambda X: X @ K, k, V, matfun=f)
    assert abs(res.mean - want.mean()) <= 1e-4 * abs(want.mean())
    np.testing.assert_allclose(res.sem, want.std() / np.sqrt(p), rtol=1e-3)
