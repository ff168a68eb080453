"""The benchmark's N > 1 path on CPU: replicas, one per rank, reduced over
the ranks -- the job's time is the slowest rank's, its simulated years all
ranks' -- and the reference arm runs on rank 0 alone.  Two gloo ranks on
127.0.0.1; no GPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=2)
    import bench
    ws, r, local = bench.dist_env()
    m = bench.max_over_ranks(0.25 + rank, "cpu")              # per-rank times (ms)
    s = bench.sum_over_ranks(10.0 * (rank + 1), "cpu")        # per-rank simulated years
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, ws, r, local, m, s))


def test_two_ranks_reduce_time_by_max_and_work_by_sum():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, (r0, ws, r, local, m, s) in enumerate(res):
        assert (r0, ws, r, local) == (rank, 2, rank, rank)
        assert m == 1.25            # the slower rank's time
        assert s == 30.0            # both ranks' work


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "3",
                                      "--warmup", "3"])
    args = bench.parse()
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""
