"""GPU tests of the serving runtime: continuous batching, resident factors, admission.

Bars: every completed request reaches backward error <= 1e-14; the same request gives
bit-identical solutions alone and inside a concurrent mix (the kernels' reductions are
ordered independently of co-resident work); repeat solves use the resident factor;
requests that can never fit the memory budget are refused, not hung.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BERR_TOL = 1e-14


def _drain(S, ids, timeout_s=120.0):
    import time

    got = {}
    t0 = time.time()
    while len(got) < len(ids) and time.time() - t0 < timeout_s:
        for c in S.poll(wait_ms=50):
            got[c["id"]] = c
    assert len(got) == len(ids), (len(got), len(ids))
    return got


def _mix():
    rng = np.random.default_rng(3)
    reqs = []
    for i in range(40):
        n = int(np.exp(rng.uniform(np.log(64), np.log(2400))))
        reqs.append(dict(n=n, matrix_seed=1000 + i, rhs_seed=5000 + i, key=i, kind=0))
    # two systems routed out of core (order >= OOC_MIN_N): FP64 factor of a host copy
    # through a small device budget, solve with the host factor
    reqs.append(dict(n=2600, matrix_seed=777, rhs_seed=778, key=100, kind=0))
    reqs.append(dict(n=2900, matrix_seed=779, rhs_seed=780, key=101, kind=0))
    # repeat solves on some of the matrices, fresh right-hand sides
    for k, i in enumerate([0, 3, 7, 11, 20, 31]):
        reqs.append(dict(n=reqs[i]["n"], matrix_seed=1000 + i, rhs_seed=9000 + k, key=i, kind=1))
    return reqs


# the out-of-core route in these tests: orders from 2500, a device panel budget of 40 tiles
OOC = dict(ooc_min_n=2500, ooc_budget=40 * 256 * 256 * 8)


def test_mix_equals_alone_and_reaches_tolerance(ooc):
    from oocdag_gb300.server import Server

    reqs = _mix()
    # alone: one request at a time (each waits for the previous to finish)
    alone = {}
    with Server(workers=4, nb=256, prec="bf16x3", batch_window_ms=0.2, **OOC) as S:
        for q in reqs:
            rid = S.submit(keep_solution=True, **q)
            c = _drain(S, [rid])[rid]
            assert c["status"] == 0 and c["info"] == 0, (c, S.last_error())
            alone[(q["key"], q["rhs_seed"])] = (S.solution(rid, q["n"]), c)
    # mix: everything submitted at once; small ones batch together, large ones overlap
    with Server(workers=4, nb=256, prec="bf16x3", batch_window_ms=2.0, **OOC) as S:
        ids = {}
        for q in reqs[:42]:
            ids[S.submit(keep_solution=True, **q)] = q
        first = _drain(S, list(ids))
        for q in reqs[42:]:  # repeats after their factors exist
            ids[S.submit(keep_solution=True, **q)] = q
        rest = _drain(S, [i for i in ids if i not in first])
        done = {**first, **rest}
        for rid, q in ids.items():
            c = done[rid]
            assert c["status"] == 0 and c["info"] == 0, (c, S.last_error())
            assert c["backward_error"] <= BERR_TOL, c
            x = S.solution(rid, q["n"])
            xa, ca = alone[(q["key"], q["rhs_seed"])]
            np.testing.assert_array_equal(x, xa)  # the same result alone and in the mix
            if q["kind"] == 1:
                assert c["factor_reused"] == 1
        paths = {c["path"] for c in done.values()}
        assert paths == {0, 1, 2}  # the batched kernel, the pipelines and the out-of-core route


def test_large_orders_mix_equals_alone(ooc):
    # Orders up to 16384 in HBM (no out-of-core route): four pipelines factor and refine them
    # side by side with a stream of small batched systems; each solution must be bit-identical
    # to the one the same request gets alone, and reach the backward-error bar.
    from oocdag_gb300.server import Server

    rng = np.random.default_rng(11)
    reqs = [dict(n=n, matrix_seed=2000 + i, rhs_seed=6000 + i, key=i, kind=0)
            for i, n in enumerate([4096, 16384, 6000, 9999, 12288, 3000, 8192, 5000])]
    reqs += [dict(n=int(rng.integers(32, 512)), matrix_seed=3000 + i, rhs_seed=7000 + i, key=100 + i, kind=0)
             for i in range(24)]
    alone = {}
    with Server(workers=4, nb=512, prec="bf16x3", batch_window_ms=0.2) as S:
        for q in reqs:
            rid = S.submit(keep_solution=True, **q)
            c = _drain(S, [rid], timeout_s=300.0)[rid]
            assert c["status"] == 0 and c["info"] == 0, (c, S.last_error())
            alone[q["key"]] = S.solution(rid, q["n"])
    with Server(workers=4, nb=512, prec="bf16x3", batch_window_ms=2.0) as S:
        ids = {S.submit(keep_solution=True, **q): q for q in reqs}
        done = _drain(S, list(ids), timeout_s=300.0)
        for rid, q in ids.items():
            c = done[rid]
            assert c["status"] == 0 and c["info"] == 0, (c, S.last_error())
            assert c["backward_error"] <= BERR_TOL, c
            np.testing.assert_array_equal(S.solution(rid, q["n"]), alone[q["key"]])
        assert {c["path"] for c in done.values()} == {0, 1}


def test_refuses_requests_that_never_fit(ooc):
    from oocdag_gb300.server import Server

    with Server(workers=2, nb=256, hbm_budget=64 << 20) as S:
        big = S.submit(n=8192, matrix_seed=1, rhs_seed=2, key=1)
        small = S.submit(n=200, matrix_seed=3, rhs_seed=4, key=2)
        got = _drain(S, [big, small])
        assert got[big]["status"] == ooc.OOC_ERR_BUDGET
        assert got[small]["status"] == 0 and got[small]["backward_error"] <= BERR_TOL


def test_eviction_then_recompute(ooc):
    from oocdag_gb300.server import Server

    # a budget that holds about one factor of n=2048: the second evicts the first, and a
    # repeat solve of the first is recomputed (not reused) yet still correct
    # (the server reserves the factor plus 64 n bytes and 64 MiB of refinement workspace)
    budget = int(ooc.factor_bytes(2048, 256, "bf16x3") * 1.5) + (64 << 20) + 64 * 2048
    with Server(workers=1, nb=256, hbm_budget=budget) as S:
        a = S.submit(n=2048, matrix_seed=11, rhs_seed=1, key=1)
        assert _drain(S, [a])[a]["status"] == 0, S.last_error()
        b = S.submit(n=2048, matrix_seed=12, rhs_seed=1, key=2)
        assert _drain(S, [b])[b]["status"] == 0, S.last_error()
        r = S.submit(n=2048, matrix_seed=11, rhs_seed=7, key=1, kind=1)
        c = _drain(S, [r])[r]
        assert c["status"] == 0 and c["factor_reused"] == 0 and c["backward_error"] <= BERR_TOL
        r2 = S.submit(n=2048, matrix_seed=11, rhs_seed=8, key=1, kind=1)
        c2 = _drain(S, [r2])[r2]
        assert c2["factor_reused"] == 1 and c2["backward_error"] <= BERR_TOL
