"""The multi-rank (replica) logic of bench.py on CPU: two gloo ranks in spawned processes.

A DMRG chain does not shard, so N ranks run N independent replicas of the timed step. The job's
step time is the slowest rank's and its rate counts every replica's flops; the reference arm runs
on rank 0 alone while the other ranks leave at once without work.
"""
import io
import multiprocessing as mp
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FLOPS = 9.47e9


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    try:
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws),
                          RANK=str(rank), LOCAL_RANK=str(rank))
        sys.path.insert(0, ROOT)
        import torch.distributed as dist

        import bench

        dist.init_process_group("gloo", rank=rank, world_size=ws)
        info = bench.dist_info()
        # replica step times differ per rank: the job's step time is the slowest one
        t, value = bench.replica_rate(0.010 * (rank + 1), FLOPS, ws, "cpu")
        # the reference arm on a rank other than 0: returns before any work, prints nothing
        out = io.StringIO()
        ref = "skipped"
        if rank != 0:
            with redirect_stdout(out):
                ref = bench.run_reference(bench.parse(["--impl", "reference", "--gpus", str(ws)]))
        dist.barrier()
        dist.destroy_process_group()
        q.put((rank, info, t, value, ref, out.getvalue()))
    except Exception as e:  # reported to the parent
        q.put((rank, "error", repr(e), None, None, None))


def _run_ranks(ws):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = {}
    try:
        for _ in range(ws):
            r = q.get(timeout=120)
            res[r[0]] = r
    finally:
        for p in procs:
            p.join(timeout=30)
            if p.is_alive():
                p.kill()
    return res


@pytest.mark.parametrize("ws", [2])
def test_replica_rate_gloo(ws):
    res = _run_ranks(ws)
    assert sorted(res) == list(range(ws))
    for rank, info, t, value, ref, out in res.values():
        assert info != "error", t
        assert info == (ws, rank, rank)
        # every rank sees the slowest rank's step time and the whole job's rate
        assert t == pytest.approx(0.010 * ws, rel=1e-12)
        assert value == pytest.approx(ws * FLOPS / (0.010 * ws) / 1e9, rel=1e-12)
        if rank != 0:
            assert ref is None and out == ""


def test_replica_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench

    t, value = bench.replica_rate(0.004, FLOPS, 1)
    assert t == 0.004
    assert value == pytest.approx(FLOPS / 0.004 / 1e9, rel=1e-15)


def test_clock_soak_runs_whole_batches_for_the_requested_time():
    sys.path.insert(0, ROOT)
    import bench

    calls = {"batch": 0, "sync": 0}
    s, n = bench.clock_soak(lambda: calls.__setitem__("batch", calls["batch"] + 1),
                            lambda: calls.__setitem__("sync", calls["sync"] + 1), 0.05, 20)
    assert s >= 0.05 and n == 20 * calls["batch"] and calls["sync"] == calls["batch"] >= 1
