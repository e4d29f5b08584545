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


def test_walk_candidates_counts_the_27_bucket_walk():
    """bench.walk_candidates (vectorised) against a direct 27-bucket walk over a small cell table that has
    negative cells and hash collisions."""
    import types
    import bench
    rng = np.random.default_rng(0)
    n, bk, cs = 500, 64, 0.1
    pos = rng.uniform(-0.3, 0.5, (n, 3)).astype(np.float32)
    M = 0xFFFFFFFF

    def key(x, y, z):
        x, y, z = x & M, y & M, z & M
        h = ((x * 19349663) & M) ^ ((y * 73856093) & M) ^ ((z * 83492791) & M)
        v = (((h << 6) & M) + (x & 63) + 4 * (y & 63) + 16 * (z & 63)) & M
        return (v & 0x7FFFFFFF) % bk

    cells = np.floor(pos / np.float32(cs)).astype(np.int64).tolist()
    keys = np.array([key(*c) for c in cells])
    order = np.argsort(keys, kind="stable")
    sk, sp = keys[order], pos[order]
    off = np.zeros((bk, 2), np.uint32)
    for k in range(bk):
        idx = np.nonzero(sk == k)[0]
        if idx.size:
            off[k] = (idx[0], idx[-1] + 1)

    class F:
        def get_params(self):
            return types.SimpleNamespace(bucket_count=bk, cell_size=cs)

        def get_field(self, name):
            return sp if name == "sorted_position" else off.reshape(-1)

    want = 0
    for c in np.floor(sp / np.float32(cs)).astype(np.int64).tolist():
        for k in range(27):
            b = key(c[0] + k % 3 - 1, c[1] + (k // 3) % 3 - 1, c[2] + k // 9 - 1)
            want += int(off[b, 1]) - int(off[b, 0])
    assert bench.walk_candidates(F()) == pytest.approx(want / n, rel=1e-12)


def test_cpu_sample_rate_steps_every_state():
    """bench.cpu_sample_rate: rounds of one oracle step per sampled state until the time bound."""
    import bench
    from pcisph_gb300 import scenes
    sc = scenes.small_dam(6, seed=2)
    pos = sc.fluid_pos.astype(np.float32)
    vel = np.zeros_like(pos)
    states = [(pos, vel), (pos + np.float32(0.001), vel)]
    rate, steps, iters = bench.cpu_sample_rate(sc, states, seconds=1e-9)
    assert steps == 1 and rate > 0 and sc.min_iters <= iters <= sc.max_iters
    rate, steps, iters = bench.cpu_sample_rate(sc, states, seconds=0.05)
    assert steps >= 1 and rate > 0


def test_gpus_flag_launches_that_many_ranks():
    """`bench.py --gpus 2` started without a launcher runs itself as two ranks (torch.distributed.run on
    127.0.0.1); the reference arm runs on rank 0 alone and reports the launch's world size."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                          "--workload", "dam32k", "--steps", "1", "--warmup", "0"],
                         capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(l) for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout
    line = lines[0]
    assert line["n_gpus"] == 2 and line["impl"] == "reference" and line["steps"] == 1
    assert line["cpu_baseline"]["cores"] == os.cpu_count()


def test_rank_launch_command():
    import bench
    cmd = bench.rank_launch_command(["--gpus", "4", "--steps", "2"], 4)
    assert cmd[1:3] == ["-m", "torch.distributed.run"]
    assert "--nproc-per-node=4" in cmd and "--master-addr=127.0.0.1" in cmd
    assert cmd[-3:] == ["--gpus", "4", "--steps", "2"][-3:] and cmd[-5].endswith("bench.py")
