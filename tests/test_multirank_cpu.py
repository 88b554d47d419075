"""The N > 1 host logic of bench.py on CPU: two ranks over gloo on 127.0.0.1.

The path runs as replicas (each rank solves the whole workload on its own GPU, no
collective on the data path); what the ranks share is the barrier around the timed
region and the max-over-ranks reduction of the elapsed time.  These tests run that logic
with world size 2, check the reduction and the whole-job throughput it feeds, and check
that the reference arm's non-zero ranks exit without work or output."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        bench.barrier(dist)
        elapsed = 1.0 + rank  # the slower rank defines the job time
        m = bench.max_over_ranks(dist, elapsed)
        v = bench.replica_throughput(ws, 1e9, 5, m)
        buf = io.StringIO()
        with redirect_stdout(buf):
            r = bench.run_reference(type("A", (), {"warmup": 0, "steps": 1})(), None, ws, rank, dist) \
                if rank != 0 else None
        bench.barrier(dist)
        q.put((rank, m, v, buf.getvalue(), r))
    finally:
        dist.destroy_process_group()


def test_two_rank_reduction_and_throughput():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    for rank, m, v, text, r in out:
        assert m == 2.0                        # max over ranks of 1.0 and 2.0
        assert v == pytest.approx(2 * 1e9 * 5 / 2.0)
        if rank != 0:
            assert text == "" and r is None     # reference arm: rank 0 alone prints


def test_single_process_paths():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(None, 3.5) == 3.5
    bench.barrier(None)
    assert bench.replica_throughput(1, 2e9, 4, 2.0) == pytest.approx(4e9)
