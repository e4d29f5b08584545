"""CPU: the bench's multi-rank arithmetic over two gloo ranks (the timed region of the slowest rank, the
whole-job value of N replicas), and its JSON contract helpers."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 100.0 + 50.0 * rank  # rank 1 is slower
    got = bench.max_over_ranks(local_ms)
    value = bench.replica_value(1_000_000 * 10, world, got)
    np.save(os.path.join(out_dir, f"r{rank}.npy"), np.array([got, value]))
    dist.destroy_process_group()


def test_max_over_ranks_and_replica_value(tmp_path):
    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    for r in range(2):
        got, value = np.load(tmp_path / f"r{r}.npy")
        assert got == 150.0                      # every rank reports the slowest rank's time
        assert value == pytest.approx(2 * 1e7 / 0.150)


def test_single_process_is_identity():
    import bench
    assert bench.max_over_ranks(12.5) == 12.5
    assert bench.replica_value(100, 1, 1000.0) == 100.0
