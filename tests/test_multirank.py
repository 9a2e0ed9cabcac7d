"""Multi-rank host logic on CPU (gloo, world_size 2 and 3): the sharded-column factorization
schedule (oocdag_gb300/shard.py) against LAPACK, its failure report, and bench.py's replica
timing helpers (barrier, max/sum over ranks)."""
import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, fn, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, init_method=f"tcp://127.0.0.1:{port}")
    try:
        q.put((rank, fn(rank, world)))
    except Exception as e:  # report to the parent
        q.put((rank, e))
    finally:
        dist.destroy_process_group()


def _run(world, fn):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, fn, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
    for r, v in out.items():
        if isinstance(v, Exception):
            raise v
    return out


def _spd(n, seed, bad=None):
    rng = np.random.default_rng(seed)
    M = rng.standard_normal((n, n))
    A = M @ M.T / n + np.eye(n)
    if bad is not None:
        A[bad, bad] = -1.0
    return A


def _shard_job(rank, world):
    from oocdag_gb300 import shard

    n, nb = 301, 64
    parts, info = shard.factor(_spd(n, 5), nb)
    return {"L": shard.assemble(parts, n, nb), "info": info, "cols": sorted(parts)}


def _shard_bad_job(rank, world):
    from oocdag_gb300 import shard

    parts, info = shard.factor(_spd(200, 6, bad=130), 48)
    return info


def _bench_job(rank, world):
    import bench

    bench.barrier(world)
    return bench.allreduce_max(float(rank + 1), world), bench.allreduce_sum(float(rank + 1), world)


@pytest.mark.parametrize("world", [2, 3])
def test_sharded_columns_match_lapack(world):
    from oocdag_gb300 import shard

    out = _run(world, _shard_job)
    n, nb = 301, 64
    L = sum(v["L"] for v in out.values())
    assert all(v["info"] == 0 for v in out.values())
    want = np.linalg.cholesky(_spd(n, 5))
    assert np.abs(L - want).max() <= 1e-12 * np.abs(want).max()
    p = shard.plan(n, nb, world)
    assert [v["cols"] for _, v in sorted(out.items())] == p.columns
    assert sorted(c for cols in p.columns for c in cols) == list(range((n + nb - 1) // nb))


def test_sharded_columns_report_lapack_info():
    import scipy.linalg as sla

    out = _run(2, _shard_bad_job)
    want = sla.lapack.dpotrf(_spd(200, 6, bad=130), lower=1)[1]
    assert set(out.values()) == {want}


def test_bench_replica_helpers_over_ranks():
    out = _run(2, _bench_job)
    assert all(v == (2.0, 3.0) for v in out.values())
