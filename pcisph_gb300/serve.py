"""Continuous-batching server of PCISPH rollouts over one batch pool (the pcisph_batch_* C ABI).

A request is a scene plus a rollout length in time steps. Requests wait in arrival order until their
device memory fits the budget (FIFO: the head of the queue blocks the rest, so no request starves);
admitted requests join the running batch at its next step, every running scene advances one time step per
batch step with its own convergence loop, and a scene leaves the batch after its last step, its final
state read back to the host. The batch compacts once per step for all scenes that left.

Reported per request: queueing delay (arrival to admission) and rollout latency (arrival to final state on
the host); per batch step: its duration. With step_timeout_ms, a batch step still running after that bound
is reported as stalled (a bounded wait on the stream, pcisph_batch_sync_for) before the server waits on;
nothing on the device is interrupted. No counterpart in the reference, which steps one scene in a
render loop (main.cpp:185-223).
"""
import math
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import scenes as _scenes
from ._lib import ERR_TIMEOUT, PcisphError


class Request:
    """A rollout request: `steps` time steps of a scene. The scene is given, or built on first use from a
    spec (kind, target particle count, aspect ratios, seed, jitter id offset), so a long queue of requests
    holds no particle arrays."""

    def __init__(self, rid, arrival, scene=None, steps=0, spec=None):
        self.rid, self.arrival, self.steps, self.spec = rid, float(arrival), int(steps), spec
        self._scene = scene

    @property
    def scene(self):
        if self._scene is None:
            kind, n, ax, az, seed, offset, d, dt = self.spec
            if kind == "dam":
                self._scene = _scenes.batch_dam(n, ax, az, d, seed, offset, dt, f"req{self.rid}")
            else:
                self._scene = _scenes.batch_drop(n, d, seed, offset, dt, name=f"req{self.rid}")
        return self._scene

    def release(self):
        """Drop a built scene's arrays (it is rebuilt, identically, if used again)."""
        if self.spec is not None:
            self._scene = None

    @property
    def particles(self):
        return self.scene.fluid_count

    @property
    def particles_bound(self):
        """An upper bound of the particle count that needs no scene (the generators stay within 20% of
        their target count; the bound allows 30%)."""
        if self.spec is None:
            return self.particles
        return int(1.3 * self.spec[1]) + 256


@dataclass
class Completion:
    rid: int
    arrival: float
    admitted: float
    finished: float
    steps: int
    particles: int
    iterations: int     # corrective iterations over the rollout
    status: int         # pcisph_step_status bits seen during the rollout
    position: np.ndarray = None
    velocity: np.ndarray = None
    unconverged_steps: int = 0      # steps that ended at the iteration cap above the scene's threshold
    max_density_error: float = 0.0  # largest end-of-step max density variation / rest density
    threshold: float = 0.01         # the scene's density variation threshold

    @property
    def latency(self):
        return self.finished - self.arrival

    @property
    def queueing(self):
        return self.admitted - self.arrival


def poisson_requests(count, rate, n_min=2048, n_max=262144, steps_min=100, steps_max=1000, seed=4, d=0.01,
                     delta_t=1e-3):
    """The serving workload: `count` requests with exponential inter-arrival times at `rate` per second,
    particle counts log-uniform in [n_min, n_max], rollouts uniform in [steps_min, steps_max]; scenes as
    the batched workload (dam-break blocks or spheres dropped into a pool), built when first used; request
    k's particles draw their jitter from ids k * 2^20 + i. Deterministic in `seed`."""
    ids = np.arange(count, dtype=np.uint64)
    u_t, u_n, u_r, u_k, u_a, u_b = (_scenes.uniform(seed, ids, a, stream=2) for a in range(6))
    arrivals = np.cumsum(-np.log1p(-u_t) / rate)
    out = []
    for k in range(count):
        n = int(round(math.exp(math.log(n_min) + u_n[k] * (math.log(n_max) - math.log(n_min)))))
        steps = steps_min + int(u_r[k] * (steps_max - steps_min + 1))
        kind = "dam" if u_k[k] < 0.5 else "drop"
        spec = (kind, n, 0.5 + 1.5 * float(u_a[k]), 0.5 + 1.5 * float(u_b[k]), seed, k << 20, d, delta_t)
        out.append(Request(k, float(arrivals[k]), steps=steps, spec=spec))
    return out


def shard(requests, rank, world):
    """Requests of one GPU when several serve one stream: request k on rank k mod world (scenes are
    independent; nothing is exchanged between GPUs)."""
    return [r for r in requests if r.rid % world == rank]


@dataclass
class _Running:
    req: Request
    sid: int
    arrived: float
    admitted: float
    left: int
    threshold: float = 0.01


@dataclass
class ServeReport:
    completions: list
    step_ms: list
    wall_s: float
    admitted: int
    rejected: list = field(default_factory=list)
    queued_at_end: int = 0
    running_at_end: int = 0
    particle_steps: int = 0
    peak_particles: int = 0
    stalled_steps: list = field(default_factory=list)  # batch-step indices that outlived step_timeout_ms

    def summary(self):
        lat = np.array([c.latency for c in self.completions]) if self.completions else np.zeros(0)
        que = np.array([c.queueing for c in self.completions]) if self.completions else np.zeros(0)
        st = np.array(self.step_ms) if self.step_ms else np.zeros(0)

        def pct(a, q):
            return float(np.percentile(a, q)) if a.size else None
        return {
            "completed": len(self.completions), "admitted": self.admitted, "rejected": len(self.rejected),
            "queued_at_end": self.queued_at_end, "running_at_end": self.running_at_end,
            "wall_s": self.wall_s, "batch_steps": len(self.step_ms),
            "particle_steps_per_s": self.particle_steps / self.wall_s if self.wall_s > 0 else 0.0,
            "scenes_per_s": len(self.completions) / self.wall_s if self.wall_s > 0 else 0.0,
            "step_ms_p50": pct(st, 50), "step_ms_p99": pct(st, 99),
            "rollout_s_p50": pct(lat, 50), "rollout_s_p99": pct(lat, 99),
            "queueing_s_p50": pct(que, 50), "queueing_s_p99": pct(que, 99),
            "peak_particles": self.peak_particles, "stalled_steps": len(self.stalled_steps),
            "accuracy_gate": accuracy_gate(self.completions),
        }


def accuracy_gate(completions):
    """The density-error gate over completed rollouts (the reference's check, Fluid.cpp:301-306, applied to
    every step): rollouts whose every step ended below the threshold, the scene-steps that ended at the
    iteration cap above it, and the largest end-of-step error seen."""
    steps = sum(c.steps for c in completions)
    capped = sum(c.unconverged_steps for c in completions)
    return {
        "rollouts_all_steps_within": sum(1 for c in completions if c.unconverged_steps == 0),
        "rollouts": len(completions),
        "scene_steps_at_cap": capped, "scene_steps": steps,
        "max_density_error": max((c.max_density_error for c in completions), default=0.0),
        "threshold": max((c.threshold for c in completions), default=0.01),
    }


class Server:
    """Admission, stepping and retirement over one batch pool.

    batch: a pcisph_gb300.Batch (or an object with its methods: add_scene, remove_scene, step, sync, stats,
    get_field). budget_bytes bounds the device memory of the admitted scenes through the batch memory
    model (bytes per particle, bytes per scene); max_particles and max_scenes are the pool's own limits.
    step_timeout_ms: report batch steps that run longer (None: no watch).
    """

    def __init__(self, batch, budget_bytes, bytes_per_particle, bytes_per_scene, max_particles, max_scenes,
                 keep_state=True, clock=time.perf_counter, step_timeout_ms=None):
        self.batch = batch
        self.budget = int(budget_bytes)
        self.bpp, self.bps = int(bytes_per_particle), int(bytes_per_scene)
        self.max_particles, self.max_scenes = int(max_particles), int(max_scenes)
        self.keep_state = keep_state
        self.clock = clock
        self.step_timeout_ms = step_timeout_ms
        self.queue = deque()     # (request, arrival time on the run's clock), arrival order
        self.running = []        # _Running, admission order
        self.used_bytes = 0
        self.used_particles = 0
        self._particles = {}     # particle count of every admitted request

    def cost(self, req):
        n = self._particles.get(req.rid)
        return (req.particles if n is None else n) * self.bpp + self.bps

    def fits_ever(self, req):
        n = req.particles_bound  # at arrival: no scene is built for a request that may wait long
        return n * self.bpp + self.bps <= self.budget and n <= self.max_particles

    def _admit(self, now):
        admitted = 0
        while self.queue:
            req, arrived = self.queue[0]
            if (self.used_bytes + self.cost(req) > self.budget or
                    self.used_particles + req.particles > self.max_particles or
                    len(self.running) >= self.max_scenes):
                break  # FIFO: the head waits for room, the others wait behind it
            self.queue.popleft()
            sid = self.batch.add_scene(req.scene)
            self.running.append(_Running(req, sid, arrived, now, req.steps, float(req.scene.threshold)))
            self.used_bytes += self.cost(req)
            self.used_particles += req.particles
            self._particles[req.rid] = req.particles
            req.release()  # the pool holds the state now
            admitted += 1
        return admitted

    def _retire(self, now):
        done, keep = [], []
        for r in self.running:
            (done if r.left == 0 else keep).append(r)
        out = []
        for r in done:
            st = self.batch.stats(r.sid)
            pos = vel = None
            if self.keep_state:
                n = self._particles[r.req.rid]
                pos = self.batch.get_field(r.sid, "position", n)
                vel = self.batch.get_field(r.sid, "velocity", n)
            self.batch.remove_scene(r.sid)
            n = self._particles.pop(r.req.rid)
            self.used_bytes -= n * self.bpp + self.bps
            self.used_particles -= n
            out.append(Completion(r.req.rid, r.arrived, r.admitted, self.clock_now(), r.req.steps,
                                  n, int(st.total_iterations), int(st.status_all), pos, vel,
                                  int(getattr(st, "unconverged_steps", 0)),
                                  float(getattr(st, "max_density_error_max", 0.0)), r.threshold))
        self.running = keep
        return out

    def clock_now(self):
        return self.clock() - self._t0

    def run(self, requests, duration=None, realtime=True):
        """Serve `requests` (sorted by arrival). realtime: requests arrive at their arrival times on the
        wall clock; otherwise all are present at the start (and latencies count from the start).
        duration bounds the wall time (seconds): no batch step starts after it. Returns a ServeReport."""
        pending = sorted(requests, key=lambda r: r.arrival)
        pi = 0
        self._t0 = self.clock()
        completions, step_ms, rejected, stalled = [], [], [], []
        admitted = particle_steps = peak = 0
        while True:
            now = self.clock_now()
            while pi < len(pending) and (not realtime or pending[pi].arrival <= now):
                req = pending[pi]
                pi += 1
                if self.fits_ever(req):
                    self.queue.append((req, req.arrival if realtime else 0.0))
                else:
                    rejected.append(req.rid)
            admitted += self._admit(now)
            if not self.running:
                if pi >= len(pending) and not self.queue:
                    break
                if duration is not None and now >= duration:
                    break
                if pi < len(pending):  # idle until the next arrival
                    time.sleep(max(0.0, min(pending[pi].arrival - now, 0.05)))
                continue
            if duration is not None and now >= duration:
                break
            t0 = self.clock()
            self.batch.step(1)
            if self.step_timeout_ms is None:
                self.batch.sync()
            else:
                try:
                    self.batch.sync(timeout_ms=self.step_timeout_ms)
                except PcisphError as e:
                    if e.code != ERR_TIMEOUT:
                        raise
                    stalled.append(len(step_ms))
                    self.batch.sync()
            step_ms.append((self.clock() - t0) * 1e3)
            particle_steps += self.used_particles
            peak = max(peak, self.used_particles)
            for r in self.running:
                r.left -= 1
            completions += self._retire(self.clock_now())
        return ServeReport(completions, step_ms, self.clock_now(), admitted, rejected, len(self.queue),
                           len(self.running), particle_steps, peak, stalled)
