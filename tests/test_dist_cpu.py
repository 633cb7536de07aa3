"""The multi-rank host logic of bench.py on CPU: two gloo ranks (127.0.0.1) set up the
process group the way torchrun's environment asks, meet at the barrier, and agree on
the max-over-ranks time that the benchmark reports (replicas: each rank times its own
copy of the workload; the slowest one sets the whole job's time)."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, ws, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(ws),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    got_ws, got_rank, _ = bench.dist_setup(None)
    bench.barrier(got_ws)
    t = bench.barrier_max(0.5 + rank, got_ws)
    out.put((got_rank, got_ws, t, dist.get_backend()))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    if torch.cuda.is_available():
        pytest.skip("the gloo path is the CPU one")
    ws = 2
    port = 29500 + os.getpid() % 1000
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1]
    assert all(r[1] == 2 and r[2] == 1.5 and r[3] == "gloo" for r in res)
