"""Multi-rank host logic of bench.py on CPU (gloo, two processes): the run is N independent
replicas (one chain per rank, no collective on the data path) whose step time is the maximum
over ranks; the reference arm runs on rank 0 only."""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, str(ROOT))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    v = bench.max_over_ranks(1.5 + rank, torch.device("cpu"))
    Path(outdir, f"r{rank}").write_text(repr(v))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    got = [float(Path(tmp_path, f"r{r}").read_text()) for r in range(world)]
    assert got == [2.5, 2.5]


def test_max_over_ranks_without_group():
    import torch

    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.25, torch.device("cpu")) == 3.25


def test_reference_arm_rank0_only(capsys, monkeypatch):
    sys.path.insert(0, str(ROOT))
    import bench

    monkeypatch.setenv("RANK", "1")
    bench.run_reference(None)  # ranks other than 0 return before reading the arguments
    assert capsys.readouterr().out == ""
