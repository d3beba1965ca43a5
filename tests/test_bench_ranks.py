"""bench.py's multi-rank logic on CPU (gloo, world size 2): every rank times its own replica, the job
time is the slowest rank's, the whole-job value counts the solves of all ranks; the reference arm runs
on rank 0 only.  No GPU: the same helpers run over NCCL under torchrun on GPUs."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out_dir):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    local = [1.25, 2.5][rank]
    total = bench.max_over_ranks(local, world, "cpu")
    value = bench.job_value(5, world, total)
    dist.destroy_process_group()
    Path(out_dir, f"r{rank}").write_text(f"{total} {value}")


def test_max_over_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    import bench

    for r in range(2):
        total, value = map(float, (tmp_path / f"r{r}").read_text().split())
        assert total == 2.5  # the slowest rank's time on every rank
        assert value == bench.NEV * 5 * 2 / 2.5


def test_single_rank_and_reference_arm_other_ranks():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.0, 1) == 3.0
    args = type("A", (), {"steps": 1, "warmup": 0, "gpus": 2})()
    assert bench.main_reference(args, 1, 2) is None  # ranks other than 0 exit without work
