"""Multi-GPU runs are replicas (one case per rank, no data-path collective); the only
cross-rank step is the job's step time, the maximum over ranks.  Checked with two gloo ranks
on the CPU (bench.replica_step_ms)."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        import bench
        out[rank] = bench.replica_step_ms(1.5 + rank, world, device='cpu')
    finally:
        dist.destroy_process_group()


def test_replica_step_time_is_the_maximum_over_ranks():
    torch = pytest.importorskip('torch')
    import torch.multiprocessing as mp
    ctx = mp.get_context('spawn')
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert dict(out) == {0: 2.5, 1: 2.5}


def test_single_rank_keeps_its_time():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replica_step_ms(3.25, 1) == 3.25
