"""CPU: the serving scheduler (admission, FIFO order, budget, retirement) over a fake batch, and request
sharding over two gloo ranks."""
import os

import numpy as np
import pytest

from pcisph_gb300 import scenes
from pcisph_gb300.serve import Request, Server, poisson_requests, shard


class FakeBatch:
    """The methods of pcisph_gb300.Batch the server uses; records what a real pool would hold."""

    class Stats:
        def __init__(self, steps):
            self.total_iterations = 3 * steps
            self.status_all = 1 if steps >= 8 else 0  # 8-step rollouts end one step at the cap
            self.unconverged_steps = 1 if steps >= 8 else 0
            self.max_density_error_max = 0.02 if steps >= 8 else 0.009

    def __init__(self, budget, bpp, bps):
        self.live = {}      # sid -> [particles, steps taken]
        self.next = 1
        self.budget, self.bpp, self.bps = budget, bpp, bps
        self.max_live_bytes = 0
        self.added = []

    def add_scene(self, scene):
        sid = self.next
        self.next += 1
        self.live[sid] = [scene.fluid_count, 0]
        self.added.append(scene.name)
        used = sum(n * self.bpp + self.bps for n, _ in self.live.values())
        assert used <= self.budget
        self.max_live_bytes = max(self.max_live_bytes, used)
        return sid

    def remove_scene(self, sid):
        del self.live[sid]

    def step(self, n=1):
        for v in self.live.values():
            v[1] += n

    def sync(self, timeout_ms=None):
        pass

    def stats(self, sid):
        return self.Stats(self.live[sid][1])

    def get_field(self, sid, name, count):
        assert count == self.live[sid][0]
        return np.full((count, 3), self.live[sid][1], np.float32)  # the steps the scene took


def _tiny_requests(count=40, seed=1):
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    for k in range(count):
        t += rng.exponential(0.001)
        sc = scenes.batch_dam(int(rng.integers(100, 400)), 1.0, 1.0, seed=seed, name=f"r{k}")
        out.append(Request(k, t, sc, int(rng.integers(2, 9))))
    return out


@pytest.mark.parametrize("realtime", [False, True])
def test_every_request_runs_exactly_its_steps_within_budget(realtime):
    reqs = _tiny_requests()
    bpp, bps = 10, 100
    budget = 6 * 400 * bpp  # a few scenes at a time
    fb = FakeBatch(budget, bpp, bps)
    srv = Server(fb, budget, bpp, bps, max_particles=10**6, max_scenes=64)
    rep = srv.run(reqs, realtime=realtime)
    assert sorted(c.rid for c in rep.completions) == [r.rid for r in reqs]
    by_id = {r.rid: r for r in reqs}
    for c in rep.completions:
        assert (c.position == by_id[c.rid].steps).all()  # stepped exactly its rollout length
        assert c.iterations == 3 * c.steps
        assert c.arrival <= c.admitted <= c.finished
    assert fb.added == [r.scene.name for r in sorted(reqs, key=lambda r: r.arrival)]  # FIFO admission
    assert 0 < fb.max_live_bytes <= budget
    assert not fb.live and rep.running_at_end == 0 and rep.queued_at_end == 0
    s = rep.summary()
    assert s["completed"] == len(reqs) and s["particle_steps_per_s"] > 0
    capped = sum(1 for r in reqs if r.steps >= 8)
    assert 0 < capped < len(reqs)
    assert s["accuracy_gate"] == {"rollouts_all_steps_within": len(reqs) - capped, "rollouts": len(reqs),
                                  "scene_steps_at_cap": capped, "scene_steps": sum(r.steps for r in reqs),
                                  "max_density_error": 0.02, "threshold": pytest.approx(0.01)}


def test_oversized_requests_are_rejected_and_scene_limit_holds():
    reqs = _tiny_requests(12)
    big = scenes.batch_dam(5000, 1.0, 1.0, name="big")
    reqs.insert(3, Request(99, reqs[2].arrival, big, 3))
    fb = FakeBatch(10**9, 1, 0)
    srv = Server(fb, 10**9, 1, 0, max_particles=2000, max_scenes=2)
    rep = srv.run(reqs, realtime=False)
    assert rep.rejected == [99]
    assert len(rep.completions) == len(reqs) - 1


def test_duration_bounds_the_run():
    reqs = _tiny_requests(5)
    for r in reqs:
        r.steps = 10**6
    fb = FakeBatch(10**9, 1, 0)
    rep = Server(fb, 10**9, 1, 0, 10**6, 64).run(reqs, duration=0.05, realtime=False)
    assert rep.completions == [] and rep.running_at_end == 5 and rep.wall_s >= 0.05


def test_poisson_requests_shape():
    reqs = poisson_requests(200, rate=200.0, seed=4)
    n = np.array([r.particles for r in reqs])
    steps = np.array([r.steps for r in reqs])
    gaps = np.diff([0.0] + [r.arrival for r in reqs])
    assert n.min() >= 0.85 * 2048 and n.max() <= 1.1 * 262144
    assert steps.min() >= 100 and steps.max() <= 1000
    assert 0.5 / 200 < gaps.mean() < 2.0 / 200
    again = poisson_requests(200, rate=200.0, seed=4)
    assert [r.arrival for r in again] == [r.arrival for r in reqs]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    reqs = shard(_tiny_requests(30, seed=7), rank, world)
    fb = FakeBatch(10**9, 1, 0)
    rep = Server(fb, 10**9, 1, 0, 10**6, 64).run(reqs, realtime=False)
    got = [None] * world
    dist.all_gather_object(got, [c.rid for c in rep.completions])
    if rank == 0:
        np.save(os.path.join(out_dir, "rids.npy"), np.array(sorted(sum(got, [])), dtype=np.int64))
        np.save(os.path.join(out_dir, "sizes.npy"), np.array([len(g) for g in got]))
    dist.destroy_process_group()


def test_requests_shard_over_two_gloo_ranks(tmp_path):
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    rids = np.load(tmp_path / "rids.npy")
    sizes = np.load(tmp_path / "sizes.npy")
    assert rids.tolist() == list(range(30))  # every request served once, by exactly one rank
    assert sizes.tolist() == [15, 15]


def test_stalled_steps_are_reported_and_waited_out():
    """step_timeout_ms: a batch step whose bounded wait times out is recorded as stalled, the server then
    waits for it, and every request still completes with its own step count."""
    from pcisph_gb300._lib import ERR_INVALID_ARG, ERR_TIMEOUT, PcisphError

    class SlowBatch(FakeBatch):
        def __init__(self, *a, slow=(), fail=None):
            super().__init__(*a)
            self.steps_done, self.slow, self.fail, self.waits = 0, set(slow), fail, []

        def step(self, n=1):
            super().step(n)
            self.steps_done += n

        def sync(self, timeout_ms=None):
            self.waits.append(timeout_ms)
            k = self.steps_done - 1
            if timeout_ms is not None and k == self.fail:
                raise PcisphError(ERR_INVALID_ARG, "not a timeout")
            if timeout_ms is not None and k in self.slow:
                raise PcisphError(ERR_TIMEOUT, "still running")

    reqs = _tiny_requests(10)
    bpp, bps = 10, 100
    budget = 4 * 400 * bpp
    fb = SlowBatch(budget, bpp, bps, slow=(1, 4))
    srv = Server(fb, budget, bpp, bps, max_particles=10**6, max_scenes=64, step_timeout_ms=250)
    rep = srv.run(reqs, realtime=False)
    assert rep.stalled_steps == [1, 4] and rep.summary()["stalled_steps"] == 2
    assert sorted(c.rid for c in rep.completions) == list(range(10))
    for c in rep.completions:
        assert c.steps == reqs[c.rid].steps and np.all(c.position == c.steps)
    assert fb.waits.count(None) == 2 and fb.waits.count(250) == len(rep.step_ms)
    # any other error of the bounded wait propagates
    fb = SlowBatch(budget, bpp, bps, fail=2)
    srv = Server(fb, budget, bpp, bps, max_particles=10**6, max_scenes=64, step_timeout_ms=250)
    with pytest.raises(PcisphError):
        srv.run(_tiny_requests(10), realtime=False)
