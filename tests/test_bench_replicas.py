"""The replica path of bench.py on CPU: two ranks over gloo (no GPU). One
solve does not shard, so under torchrun every rank runs its own replica and
rank 0 reports the max of the ranks' times; the reference arm runs on rank 0
only and the other ranks exit without work."""

import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, ws: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    try:
        r, w = bench._dist()
        assert (r, w) == (rank, ws)
        bench._barrier(w)
        worst = bench._max_over_ranks(0.5 + rank, w)            # each rank's own step time
        ref = bench.run_reference(None, r, w) if r != 0 else "rank 0 runs"
        bench._barrier(w)
        q.put((rank, worst, ref))
    finally:
        if dist.is_initialized():
            dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    codes = [p.exitcode for p in procs]
    for p in procs:
        if p.is_alive():
            p.kill()
    assert codes == [0, 0], f"rank exit codes {codes}"
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert [g[1] for g in got] == [pytest.approx(1.5), pytest.approx(1.5)]
    assert got[1][2] is None                                     # rank 1: no reference work
