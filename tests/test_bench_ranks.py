"""The bench's multi-rank host logic on CPU, world size 2 over gloo: the job's
time is the slowest rank's and its work the sum of the ranks' (replicas:
every rank renders its own frame, no data-path collective), and the
reference arm runs on rank 0 alone. No GPU needed."""
import contextlib
import io
import os
import socket
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # per rank: device time (ms), rays, samples; then an e2e pair
        mine = torch.tensor([10.0 + 5.0 * rank, 1000.0 * (rank + 1), 7.0 * (rank + 1)], dtype=torch.float64)
        e2e = torch.tensor([0.5 + 0.25 * rank, 300.0 + rank], dtype=torch.float64)
        out.put((rank, bench.reduce_over_ranks(mine, 1, world), bench.reduce_over_ranks(e2e, 1, world)))
    finally:
        dist.destroy_process_group()


def test_reduce_over_two_gloo_ranks():
    pytest.importorskip("torch.distributed")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, head, e2e in got:
        # time: the slower rank; work: both ranks' together
        assert head == [15.0, 3000.0, 21.0], (rank, head)
        assert e2e == [0.75, 601.0], (rank, e2e)


def test_single_rank_keeps_its_values():
    import torch

    import bench
    assert bench.reduce_over_ranks(torch.tensor([2.0, 3.0], dtype=torch.float64), 1, 1) == [2.0, 3.0]


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun every rank starts the reference arm; ranks other than 0
    leave at once, without work or output."""
    import bench

    class Args:
        steps = 1
        warmup = 0
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference(Args(), 1, 2)
    assert buf.getvalue() == ""
