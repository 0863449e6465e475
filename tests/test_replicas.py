"""The N > 1 bench path (independent replicas; no collective on the data path): every rank runs the same
product on its own GPU, and the whole-job value is all ranks' bytes over the slowest rank's
time.  Checked here with two gloo ranks on the CPU (no GPU): the max-over-ranks reduction and
the value every rank computes."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_path):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    own_ms = [2.0, 5.0][rank]  # rank 1 is the slow one
    value, max_ms = bench.replica_value(own_ms, world, nbytes=1e9, steps=10, device=torch.device("cpu"))
    dist.barrier()
    with open(f"{out_path}.{rank}", "w") as f:
        f.write(f"{value} {max_ms}\n")
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    out = str(tmp_path / "rank")
    mp.start_processes(_rank_main, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    results = [open(f"{out}.{r}").read().split() for r in range(2)]
    for value, max_ms in results:
        assert float(max_ms) == 5.0
        # 2 ranks x 10 steps x 1 GB over 5 ms
        assert abs(float(value) - 2 * 10 * 1e9 / 5e-3 / 1e9) < 1e-6


def test_single_rank_is_its_own_time():
    torch = pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench
    value, max_ms = bench.replica_value(4.0, 1, nbytes=2e9, steps=3, device=torch.device("cpu"))
    assert max_ms == 4.0 and abs(value - 3 * 2e9 / 4e-3 / 1e9) < 1e-6


def test_cpu_legs_take_the_whole_host(monkeypatch):
    """Under torchrun OMP_NUM_THREADS is 1; the CPU legs (run on rank 0 alone) still use every
    CPU the process may run on."""
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("OMP_NUM_THREADS", "1")
    want = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    assert bench.host_threads() == want >= 1
