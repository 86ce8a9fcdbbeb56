"""bench.py --gpus N runs one independent replica per rank (the SODA sweep
does not shard: every rank runs its own job on its own seeded data).  The
host logic that turns per-rank timings into the job's line is checked here
with two gloo ranks on the CPU: the timed region is the maximum over ranks,
the units are the sum over ranks, and each rank draws its own data seed."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, ws, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(ws), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    from sodabayes_gb300 import synth
    r, w = bench._dist_init()
    bench._barrier(w)
    t_max = bench._max_over_ranks(10.0 + 5.0 * r, w)       # rank 1 is the slow one
    units = bench._sum_over_ranks(16.0 * (r + 1), w)
    spec = synth.CONFIGS[bench.SPEC_KEY]
    seed = spec.seed + 1000 * r                              # bench_ours' per-rank data seed
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, w, t_max, units, seed))


def test_replica_aggregation_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2, 2]
    assert all(o[2] == 15.0 for o in out)           # max over ranks
    assert all(o[3] == 48.0 for o in out)           # 16 + 32 units
    assert out[0][4] != out[1][4]                   # independent data per replica
