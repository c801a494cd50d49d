"""The benchmark's multi-replica logic on CPU: two gloo ranks (127.0.0.1)
aggregate their timings (slowest rank, sum of units) the way
`torchrun --nproc-per-node N bench.py --gpus N` does on GPUs, and the
reference arm runs on rank 0 only."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r took (100 + 50 r) ms for (1 + r) * 1e9 updates
    value, ms = bench.aggregate(100.0 + 50.0 * rank, (1 + rank) * 1e9, world)
    out[rank] = (value, ms)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_whole_job():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    # slowest rank: 150 ms; all units: 3e9 -> 20 G per second, the same on both ranks
    assert res[0] == res[1]
    value, ms = res[0]
    assert ms == 150.0
    assert value == pytest.approx(3e9 / 0.150 / 1e9)


def test_single_process_needs_no_process_group():
    import bench
    value, ms = bench.aggregate(200.0, 4e9, 1)
    assert ms == 200.0 and value == pytest.approx(20.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    """Under torchrun every rank but 0 exits at once without output."""
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    buf = io.StringIO()
    with redirect_stdout(buf):
        assert bench.run_reference(None) is None
    assert buf.getvalue() == ""
