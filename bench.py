"""Benchmark of the PCISPH time step on GB300: particle-steps/s at 1,048,576 particles.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on stdout (rank 0). The workload is the 1M-particle dam break: a 128 x 128 x 64 jittered
lattice (d = 0.005 m, h = 0.01 m, m = rho0 d^3), dt = 2.5e-4 s, rho0 = 1000, mu = 0.2 Pa s,
gamma = 0.5, g = -9.81, reflecting walls (restitution 0.5) in [0,1.6]x[0,1.2]x[0,0.8] m, 3..50 corrective
iterations until the max density error is below 1%. A "step" is one full PCISPH time step.

  value     N x K / sum of the K steps' device times (CUDA events on the step's stream), state resident in
            HBM, a 256 MB buffer written between timed steps (L2 flush, not timed)
  e2e       the same metric through the C ABI with pinned host buffers: each step uploads positions and
            velocities, steps, and reads both back
  roofline  the dominant kernel (largest share of a per-kernel CUDA-event pass over the same state)
  cpu_baseline  the oracle (CPU port of the reference step) on all host cores, from the same state
  --impl reference  the reference's CPU implementation (the oracle port; the OpenCL runtime the reference
            needs does not exist on these machines) timed on the host cores on the same workload
With --gpus N > 1 every rank runs its own replica (the step does not shard); value is summed. Started
without a launcher, --gpus N > 1 runs this script as N ranks under torch.distributed.run itself.
"""
import argparse
import json
import os
import signal
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic bytes per particle per launch (12 B per 3-vector, 4 B per scalar, the cell table amortised
# at 4 B per particle): compulsory reads and writes of each fused kernel
ALGO_BYTES = {
    "density": 20,          # x 12 + cell table 4 + rho 4
    "normal": 32,           # x 12 + rho 4 + cell table 4 + n 12
    "force": 72,            # x, v, n 36 + rho 4 + cell table 4 + F_o 12 + p 4 + x* 12
    "pressure": 40,         # x 12 + x* 12 + p 4 + cell table 4 + p 4 + err 4
    "pressure_force": 72,   # x 12 + p 4 + rho 4 + cell table 4 + F_p 12; predict: v 12, F_o 12, x* 12
    "reorder": 60,          # keys 4 + ids 4 + x, v gathered 24 + x, v written 24 + table 4
    "hash": 20,             # x 12 + key 4 + id 4
    "radix_sort": 32,       # 2 passes (10-bit digits for the 19-bit keys at 1M) of 8 B read + 8 B written
}
# compulsory bytes of a whole step per particle: 340 + 136 per corrective iteration (hash 20, 3 sort passes
# 60, cell reset 4, reorder 60, density 20, normal 32, force 72, integrate 72; per iteration predict 60,
# pressure 40, pressure force 36), vectors at their 12-byte payload
STEP_FIXED_BYTES = 340
CPU_POINTS = 8  # states of the timed run the CPU baseline samples from
STEP_ITER_BYTES = 136
DAM_WORKLOADS = {
    "dam1m": ("dam_break_1m", "particle-steps/s @1M (<=1% rho err)",
              "dam break 128x128x64 = 1,048,576 particles, d=0.005 m, dt=2.5e-4 s, reflecting walls, "
              "3-50 corrective iterations to <1% density error"),
    "dam32k": ("dam_break_32k", "particle-steps/s @32K (<=1% rho err)",
               "dam break 32^3 = 32,768 particles, d=0.02 m, dt=1e-3 s, reflecting walls, "
               "3-50 corrective iterations to <1% density error"),
    "dam1m_boundary": ("dam_break_1m_boundary", "particle-steps/s @1M with 284K boundary particles (3-7 iterations)",
                       "dam break 128x128x64 = 1,048,576 particles against 284,192 boundary particles (2 layers "
                       "lining a 1.28x0.96x0.32 m box), d=0.005 m, dt=2.5e-4 s, reflecting walls, the reference's "
                       "3-7 corrective iterations (threshold 1%)"),
    "dam8m": ("two_blocks_8m", "particle-steps/s @8M (3-50 iterations; the scene ends every step at the cap)",
              "two 256x128x128 blocks = 8,388,608 particles, d=0.0025 m, dt=1.25e-4 s, reflecting walls, "
              "3-50 corrective iterations to <1% density error"),
}
WORKLOAD = ("dam break 128x128x64 = 1,048,576 particles, d=0.005 m, dt=2.5e-4 s, reflecting walls, "
            "3-50 corrective iterations to <1% density error")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: the workload's own length -- dam1m 500, dam32k 1000, dam8m 200, "
                         "scenes 500)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="bound of the CPU baseline sample")
    ap.add_argument("--variant", type=int, default=2, help="neighbour-sweep kernel variant (pcisph_options)")
    ap.add_argument("--workload", default="dam1m",
                    choices=["dam1m", "dam1m_boundary", "dam32k", "dam8m", "scenes", "serve"],
                    help="dam1m: the 1M-particle dam break (the headline); dam32k / dam8m: the 32K and 8M "
                         "dam breaks; scenes: 256 scenes batched vs "
                         "stepped one context each; serve: Poisson requests through the serving loop")
    ap.add_argument("--requests", type=int, default=20000, help="request count of --workload serve")
    ap.add_argument("--rate", type=float, default=200.0, help="arrivals per second of --workload serve")
    ap.add_argument("--budget-gb", type=float, default=100.0, help="device memory budget of --workload serve")
    ap.add_argument("--duration", type=float, default=120.0, help="wall-time bound (s) of --workload serve")
    ap.add_argument("--scenes", type=int, default=256, help="scene count of --workload scenes")
    ap.add_argument("--scenes-leg-steps", type=int, default=20,
                    help="the 1M dam break's line also times the 256 batched scenes over this many steps after 3 "
                         "warm-up steps (batched_scenes); 0: skip")
    ap.add_argument("--autotune", action="store_true",
                    help="run the library's autotuner on the warmed-up state before timing (results unchanged)")
    ap.add_argument("--loop-mode", type=int, default=0, choices=[0, 2],
                    help="corrective loop: 0 graph WHILE node, 2 persistent cooperative kernel")
    ap.add_argument("--list-skin", type=float, default=None,
                    help="list skin in units of h: pcisph_options.list_skin of the dam-break workloads (default "
                         "0.25), a fixed skin for the batched workloads (default: each scene adapts its own)")
    ap.add_argument("--spatial-order", type=int, default=2, choices=[0, 1, 2],
                    help="pcisph_options.spatial_order of the dam-break workloads (2: the library's choice)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"dam1m": 500, "dam1m_boundary": 500, "dam32k": 1000, "dam8m": 200,
                      "scenes": 500}.get(args.workload, 200)
    return args


def free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_launch_command(argv, n):
    """The command that runs this script with arguments argv as n ranks of one node (torch.distributed.run,
    rendezvous on 127.0.0.1)."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
            "--master-addr=127.0.0.1", f"--master-port={free_port()}", os.path.abspath(__file__), *argv]


def relaunch_as_ranks(args, argv):
    """--gpus N > 1 outside a launcher (no WORLD_SIZE): run N ranks and return their exit status; None when
    this process is already a rank or N = 1."""
    if args.gpus <= 1 or "WORLD_SIZE" in os.environ:
        return None
    return subprocess.call(rank_launch_command(argv, args.gpus))


def max_over_ranks(x):
    """The largest of every rank's x (the timed region of the slowest rank); x itself on one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, world, max_ms):
    """Whole-job throughput of `world` replicas that each processed units_per_rank in at most max_ms."""
    return units_per_rank * world / (max_ms / 1e3)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_records(variant):
    """Per-kernel ncu figures of one kernel variant from the committed summary (profiles/ncu_traffic.txt):
    {kernel: {"dram_bytes_per_particle": ..., "l1tex_throughput_active_pct": ..., ...}}."""
    out = {}
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return out
    with open(path) as f:
        for line in f:
            if line.startswith("kernel="):
                kv = dict(tok.split("=", 1) for tok in line.split())
                if int(kv.get("variant", -1)) == variant:
                    out[kv["kernel"]] = {k: float(v) for k, v in kv.items()
                                         if k not in ("kernel", "variant", "source")}
    return out


def binding_unit(variant, kernel):
    """The unit that bounds a neighbour sweep by its committed ncu capture: the list sweeps gather ~24
    sectors per warp request and keep the L1 data pipe busy, not HBM."""
    r = ncu_records(variant).get(kernel, {})
    if "l1tex_throughput_active_pct" not in r:
        return None
    return {"unit": "L1/tex (gather wavefronts)", "busy_frac_while_active": r["l1tex_throughput_active_pct"] / 100.0,
            "issue_busy_frac": r.get("issue_active_pct", 0.0) / 100.0,
            "source": "profiles/ncu_traffic.txt (ncu --set full of the same kernel)"}


def ncu_traffic(variant):
    """Per-kernel DRAM bytes per particle of one kernel variant (profiles/ncu_traffic.txt)."""
    return {k: r["dram_bytes_per_particle"] for k, r in ncu_records(variant).items()
            if "dram_bytes_per_particle" in r}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the benchmark runs."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.proc, self.path, self.gpu = None, None, gpu

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.send_signal(signal.SIGTERM)
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "reasons": reasons, "samples": len(rows)}


def host_link_rates(nbytes, reps=10):
    """Pinned host <-> device copy rates (GB/s) for nbytes, the bound of the e2e copies."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        d.copy_(h, non_blocking=True)
        h.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        d.copy_(h, non_blocking=True)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(reps):
        h.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return {"h2d": reps * nbytes / (t1 - t0) / 1e9, "d2h": reps * nbytes / (t2 - t1) / 1e9}


def walk_candidates(f):
    """Mean candidates per particle of the reference's 27-bucket walk (grid_utils.cl:65-79) at the last
    step's sorted positions: the pair evaluations each of its neighbour sweeps makes per particle."""
    import numpy as np
    p = f.get_params()
    pos = f.get_field("sorted_position").astype(np.float32)
    off = f.get_field("cell_offsets").reshape(-1, 2).astype(np.int64)
    lens = np.maximum(off[:, 1] - off[:, 0], 0)
    bk = np.uint64(p.bucket_count)
    cell = np.floor(pos / np.float32(p.cell_size)).clip(-2.0 ** 31, 2.0 ** 31 - 1).astype(np.int64)
    total = np.zeros(pos.shape[0], np.int64)
    m32 = np.int64(0xFFFFFFFF)
    for k in range(27):
        x = (cell[:, 0] + (k % 3 - 1)) & m32
        y = (cell[:, 1] + ((k // 3) % 3 - 1)) & m32
        z = (cell[:, 2] + (k // 9 - 1)) & m32
        h = ((x * 19349663) & m32) ^ ((y * 73856093) & m32) ^ ((z * 83492791) & m32)
        v = (((h << 6) & m32) + (x & 63) + 4 * (y & 63) + 16 * (z & 63)) & m32
        key = ((v & 0x7FFFFFFF).astype(np.uint64) % bk).astype(np.int64)
        total += lens[key]
    return float(total.mean()) if total.size else 0.0


def _oracle_for(scene):
    """The oracle, the scene's parameters (boundary particles included) and step options."""
    from oracle.oracle import get as get_oracle
    from oracle.oracle import make_options
    O = get_oracle()
    p = O.derive_params(scene.particle_radius, scene.rest_density, scene.fluid_count, scene.boundary_count,
                        scene.delta_t, scene.gravity, scene.viscosity_constant(), scene.surface_tension)
    opts = make_options(threshold=scene.threshold, min_iters=scene.min_iters, max_iters=scene.max_iters,
                        walls=scene.walls, box_lo=scene.box_lo, box_hi=scene.box_hi, restitution=scene.restitution)
    return O, p, opts


def oracle_threads():
    """The OpenMP threads the oracle's loops ran on (the cores the CPU baseline used)."""
    from oracle.oracle import get as get_oracle
    return get_oracle().num_threads()


def cpu_step_rate(scene, pos, vel, seconds, max_steps=None):
    """Oracle steps from (pos, vel) until `seconds` of step time; returns (particle-steps/s, steps, iters).
    Boundary particles are sorted in the first step only, as the GPU context sorts them once."""
    import numpy as np
    O, p, opts = _oracle_for(scene)
    s = O.new_state(p, pos, vel, scene.boundary_pos)
    t_total, steps, iters = 0.0, 0, []
    while t_total < seconds and (max_steps is None or steps < max_steps):
        t0 = time.perf_counter()
        st = O.step(p, opts, s, boundary_sort=steps == 0)
        t_total += time.perf_counter() - t0
        steps += 1
        iters.append(st.iterations)
    return scene.fluid_count * steps / t_total, steps, float(np.mean(iters)), s


def cpu_sample_rate(scene, states, seconds, max_steps=None):
    """Oracle steps from each of `states` ((pos, vel) at evenly spaced points of a run) in rounds, one step
    per state per round, until `seconds` of step time or `max_steps` steps (the run's length: each state
    then covers its own segment of the run); returns (particle-steps/s, steps, mean iterations). Each run
    sorts the boundary particles in its first step (included in the time: ~2% at 284K boundary particles)."""
    import numpy as np
    O, p, opts = _oracle_for(scene)
    runs = [O.new_state(p, pos, vel, scene.boundary_pos) for pos, vel in states]
    first = [True] * len(runs)
    t_total, steps, iters = 0.0, 0, []
    while t_total < seconds and (max_steps is None or steps < max_steps):
        for k, s in enumerate(runs):
            t0 = time.perf_counter()
            st = O.step(p, opts, s, boundary_sort=first[k])
            t_total += time.perf_counter() - t0
            first[k] = False
            steps += 1
            iters.append(st.iterations)
            if t_total >= seconds or (max_steps is not None and steps >= max_steps):
                break
    return scene.fluid_count * steps / t_total, steps, float(np.mean(iters))


REFERENCE_TIMED_SECONDS = 120.0  # bound of the reference arm's timed steps (its warm-up steps are not bounded)


def reference_arm(args, rank, world):
    """The reference's CPU implementation of the step (the oracle port) on all host cores: args.warmup
    untimed steps from the workload's initial state, then up to args.steps timed steps, stopping after
    REFERENCE_TIMED_SECONDS. Under N ranks rank 0 alone runs it (with every core: a launcher's
    OMP_NUM_THREADS=1 is overridden before the oracle library loads) and the other ranks exit."""
    if rank != 0:
        return
    cores = os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(cores)
    from pcisph_gb300 import scenes
    import numpy as np
    cfg, metric, workload = DAM_WORKLOADS.get(args.workload, DAM_WORKLOADS["dam1m"])
    sc = getattr(scenes, cfg)()
    pos, vel = sc.fluid_pos, np.zeros_like(sc.fluid_pos)
    w = args.warmup
    if w:
        _, _, _, s = cpu_step_rate(sc, pos, vel, float("inf"), max_steps=w)
        pos, vel = s["f_pos"], s["f_vel"]
    rate, steps, iters, _ = cpu_step_rate(sc, pos, vel, REFERENCE_TIMED_SECONDS, max_steps=args.steps)
    cores = oracle_threads()
    line = {
        "impl": "reference", "metric": metric, "value": rate,
        "unit": "particle-steps/s", "n_gpus": world, "steps": steps, "warmup": w,
        "ms_per_step": 1e3 * sc.fluid_count / rate,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded jittered lattice)",
        "config": {"workload": workload, "particles": sc.fluid_count, "mean_iterations": iters,
                   "particle_iterations_per_s": rate * iters},
        "cpu_baseline": {"value": rate, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{sc.fluid_count} particles x {steps} steps after {w} warm-up steps "
                                   f"(oracle/pcisph_oracle.cpp, OpenMP over particles on {cores} threads; the "
                                   f"reference's OpenCL runtime is unavailable on this box)"},
        "e2e": {"value": rate, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


SCENES_WORKLOAD = ("256 scenes, particle counts log-uniform in [4,096, 131,072] (seed 3), each a dam-break block "
                   "(aspect ratios U[0.5, 2]) or a sphere dropped 0.5 m into a pool holding 30% of its particles; "
                   "d=0.01 m, dt=1e-3 s, reflecting walls, 3-50 corrective iterations to <1% density error per scene")


def scenes_workload(args, rank, world, local, emit=True, cpu_leg=True):
    """256 independent scenes: one batched step (pcisph_batch_*) against one context per scene, stepped one
    after another on the same stream. Scenes shard across ranks (scene k on rank k mod N). Prints the line
    (emit) and returns it on rank 0; cpu_leg: time the oracle on the smallest scenes too."""
    import numpy as np
    import torch
    import torch.distributed as dist

    from pcisph_gb300 import Batch, Fluid, build, scenes, setup_scene
    build.build()
    all_sc = scenes.batch_scenes(count=args.scenes)
    sc = all_sc[rank::world]
    n_total = sum(s.fluid_count for s in sc)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sampler = ClockSampler(local)
    sampler.start()

    def timed(step_fn, steps):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        for k in range(steps):
            starts[k].record(stream)
            step_fn()
            ends[k].record(stream)
        torch.cuda.synchronize()
        return max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(starts, ends)))

    # batched: every scene in one pool, one graph launch per step
    bt = Batch(local, max_particles=n_total, max_scenes=len(sc), stream=stream.cuda_stream, loop_mode=args.loop_mode)
    bt.set_list_skin("adaptive" if args.list_skin is None else args.list_skin)
    ids = [bt.add_scene(s) for s in sc]
    for _ in range(args.warmup):
        bt.step(1)
    bt.sync()
    tuned = bt.autotune(steps=2) if args.autotune else None
    snap = [(bt.get_field(i, "position", s.fluid_count), bt.get_field(i, "velocity", s.fluid_count))
            for i, s in zip(ids, sc)]
    st0 = [bt.stats(i) for i in ids]
    launches0 = bt.kernel_launches()
    ms_batch = timed(lambda: bt.step(1), args.steps)
    st1 = [bt.stats(i) for i in ids]
    launches = bt.kernel_launches() - launches0
    iters = [(b.total_iterations - a.total_iterations) / args.steps for a, b in zip(st0, st1)]
    batch_loop_iters = max(iters)
    capped = [int(b.unconverged_steps - a.unconverged_steps) for a, b in zip(st0, st1)]
    worst = int(np.argmax(capped))
    worst_state = (bt.get_field(ids[worst], "position", sc[worst].fluid_count),
                   bt.get_field(ids[worst], "velocity", sc[worst].fluid_count)) if capped[worst] else None

    # per-kernel CUDA events over the first timed steps again (profiled host-driven steps, same kernels)
    for i, (p, v) in zip(ids, snap):
        bt.set_state(i, p, v)
    prof_steps = min(args.steps, 20)
    sp0 = [bt.stats(i) for i in ids]
    bt.profile(True)
    bt.step(prof_steps)
    prof = bt.profile_read()
    bt.profile(False)
    sp1 = [bt.stats(i) for i in ids]
    # particle-iterations of the profiled steps: the pressure sweeps' work
    p_iters = sum(s.fluid_count * (b.total_iterations - a.total_iterations) for s, a, b in zip(sc, sp0, sp1))
    tot_ms = sum(ms for _, ms in prof.values())
    kernels = {k: {"launches": l, "avg_us": 1e3 * ms / l, "share": ms / tot_ms} for k, (l, ms) in prof.items()}
    roof = None
    if "pressure" in prof:
        peak, peak_kind = peaks()
        l, ms = prof["pressure"]
        achieved = ALGO_BYTES["pressure"] * p_iters / (ms / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": "pressure", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                "algo_bytes_per_particle": ALGO_BYTES["pressure"], "avg_launch_us": 1e3 * ms / l,
                "note": "algorithmic bytes of the particle-iterations of the profiled steps over the total time "
                        "of their pressure sweeps (finished scenes skip)"}

    # e2e through the batch ABI: host state of every scene in, one step, every scene's state out
    e2e_steps = min(args.steps, 5)
    pin = [(torch.empty((s.fluid_count, 3), dtype=torch.float32, pin_memory=True).numpy(),
            torch.empty((s.fluid_count, 3), dtype=torch.float32, pin_memory=True).numpy()) for s in sc]
    for (p, v), (p0, v0) in zip(pin, snap):
        p[:] = p0
        v[:] = v0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for i, (p, v) in zip(ids, pin):
            bt.set_state(i, p, v)
        bt.step(1)
        for i, s, (p, v) in zip(ids, sc, pin):
            p[:] = bt.get_field(i, "position", s.fluid_count)
            v[:] = bt.get_field(i, "velocity", s.fluid_count)
    e2e_s = time.perf_counter() - t0
    bt.close()

    # one context per scene, from the same state, each stepped once per step (graph launch each)
    ctxs = []
    for s, (p, v) in zip(sc, snap):
        f = Fluid(local, stream=stream.cuda_stream)
        setup_scene(f, s, kernel_variant=args.variant)
        f.set_fluid_state(p, v)
        ctxs.append(f)

    def step_all():
        for f in ctxs:
            f.update()
    ms_single = timed(step_all, args.steps)
    single_launches = sum(f.kernel_launches() for f in ctxs)
    for f in ctxs:
        f.close()
    clocks = sampler.stop()

    gate = {"threshold": max(s.threshold for s in sc), "scene_steps_at_cap": sum(capped),
            "scene_steps": len(sc) * args.steps, "scenes_with_capped_steps": sum(1 for c in capped if c),
            "max_density_error": max(b.max_density_error_max for b in st1),
            "max_density_error_note": "largest end-of-step error of any scene over the warm-up and timed steps",
            "worst_scene": None}
    if worst_state is not None:
        gate["worst_scene"] = capped_scene_vs_oracle(sc[worst], worst_state, capped[worst], local, stream)
    cpu = None
    if rank == 0 and world == 1 and cpu_leg:  # oracle on the smallest scenes, from the same state, bounded
        order = np.argsort([s.fluid_count for s in sc])[:8]
        done, t_cpu, cs = 0, 0.0, 0
        for k in order:
            r, steps_k, _, _ = cpu_step_rate(sc[k], snap[k][0], snap[k][1], args.cpu_seconds / 8, max_steps=args.steps)
            done += sc[k].fluid_count * steps_k
            t_cpu += sc[k].fluid_count * steps_k / r
            cs += steps_k
        cpu = {"value": done / t_cpu, "unit": "particle-steps/s", "cores": oracle_threads(), "kind": "port",
               "sample": f"the 8 smallest scenes, {cs} scene-steps from the timed loop's start state "
                         f"(oracle/pcisph_oracle.cpp with OpenMP)"}
    if rank == 0:
        n_all = sum(s.fluid_count for s in all_sc)
        value = n_all * args.steps / (ms_batch / 1e3)
        line = {
            "metric": "particle-steps/s, 256 scenes batched", "value": value, "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_batch / args.steps,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scenes)",
            "config": {"workload": SCENES_WORKLOAD, "scenes": len(all_sc), "particles": n_all,
                       "parallelism": f"scenes sharded over {world} GPU(s)",
                       "scene_steps_per_s": len(all_sc) * args.steps / (ms_batch / 1e3),
                       "mean_scene_iterations": float(np.mean(iters)), "batch_loop_iterations": batch_loop_iters,
                       "loop_mode": args.loop_mode, "autotuned": tuned,
                       "list_skin": "adaptive" if args.list_skin is None else args.list_skin,
                       "l2": "working set ~6 GB > L2"},
            "per_scene_contexts": {"value": n_all * args.steps / (ms_single / 1e3), "unit": "particle-steps/s",
                                   "ms_per_step": ms_single / args.steps, "gpu_launches": single_launches,
                                   "speedup_of_batch": ms_single / ms_batch},
            "e2e": {"value": n_total * e2e_steps * world / e2e_s, "unit": "particle-steps/s",
                    "h2d_bytes_per_step": 24 * n_total, "d2h_bytes_per_step": 24 * n_total, "steps": e2e_steps},
            "gpu_launches": launches, "roofline": roof, "kernels": kernels, "cpu_baseline": cpu, "clocks": clocks,
            "accuracy_gate": gate,
        }
        if emit:
            print(json.dumps(line), flush=True)
        return line
    return None


def capped_scene_vs_oracle(scene, state, capped_steps, device, stream):
    """The scene whose batched steps most often ended at the iteration cap, stepped once more from its state
    after the timed steps: through the oracle (the reference's step on the CPU) and through one context of its
    own, so that the line shows whether the reference's formulation also stops at the cap there."""
    from pcisph_gb300 import Fluid, setup_scene
    pos, vel = state
    O, p, opts = _oracle_for(scene)
    s = O.new_state(p, pos, vel, scene.boundary_pos)
    so = O.step(p, opts, s)
    f = Fluid(device, stream=stream.cuda_stream)
    setup_scene(f, scene)
    f.set_fluid_state(pos, vel)
    f.update()
    sg = f.stats()
    f.close()
    return {"scene": scene.name, "particles": scene.fluid_count, "batched_steps_at_cap": capped_steps,
            "max_iterations": scene.max_iters,
            "next_step_oracle": {"iterations": so.iterations, "max_density_error": so.max_err / p.rest_density},
            "next_step_gpu_alone": {"iterations": sg.iterations, "max_density_error": sg.max_density_error}}


SERVE_WORKLOAD = ("Poisson arrivals; particle counts log-uniform in [2,048, 262,144], rollouts U[100, 1000] steps, "
                  "scenes as the batched workload (seed 4); FIFO admission against a device-memory budget")


def serve_workload(args, rank, world, local):
    """The serving loop on live arrivals, bounded by --duration seconds of wall time. Requests shard over
    ranks (request k on rank k mod N); each rank serves its share on its own pool."""
    import torch
    import torch.distributed as dist

    from pcisph_gb300 import Batch, build
    from pcisph_gb300.batch import memory_model
    from pcisph_gb300.serve import Server, poisson_requests, shard
    build.build()
    # arrivals past the wall-time bound never reach the server: generate those that can
    horizon = min(args.requests, int(args.rate * args.duration * 1.2) + 16)
    reqs = shard(poisson_requests(horizon, args.rate, seed=4), rank, world)
    bpp, bps = memory_model()
    budget = int(args.budget_gb * (1 << 30))
    max_particles = min(budget // bpp, (1 << 31) - 1)
    max_scenes = min(65535, max(16, budget // (2048 * bpp + bps)))
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    bt = Batch(local, max_particles=max_particles, max_scenes=max_scenes, stream=stream.cuda_stream,
               loop_mode=args.loop_mode)
    bt.set_list_skin("adaptive" if args.list_skin is None else args.list_skin)
    srv = Server(bt, budget, bpp, bps, max_particles, max_scenes, keep_state=True)
    # warm-up: one small request served to completion before the clock starts (graph build, first launches)
    Server(bt, budget, bpp, bps, max_particles, max_scenes, keep_state=False).run(reqs[:1], realtime=False)
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        dist.barrier()
    rep = srv.run(reqs, duration=args.duration, realtime=True)
    clocks = sampler.stop()
    summ = rep.summary()
    summ["graph_instantiations"], summ["graph_updates"] = bt.graph_stats()
    bt.close()
    # the same request mix stepped as one context per request against one batch of those requests
    summ["per_scene_vs_batched"] = request_mix_comparison(reqs[:SERVE_MIX_SCENES], SERVE_MIX_STEPS, local, stream)
    if world > 1:
        got = [None] * world
        dist.all_gather_object(got, summ)
    else:
        got = [summ]
    if rank == 0:
        wall = max(g["wall_s"] for g in got)
        ps = sum(g["particle_steps_per_s"] * g["wall_s"] for g in got)
        sample = poisson_requests(min(horizon, 5000), args.rate, seed=4)
        offered = sum(r.spec[1] * r.steps for r in sample) / len(sample) * args.rate  # target counts
        line = {
            "metric": "particle-steps/s served", "value": ps / wall, "unit": "particle-steps/s", "n_gpus": world,
            "steps": summ["batch_steps"], "warmup": 1, "ms_per_step": summ["step_ms_p50"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scenes, Poisson arrivals)",
            "config": {"workload": SERVE_WORKLOAD, "rate_per_s": args.rate, "budget_gb": args.budget_gb,
                       "duration_s": args.duration, "requests_generated": horizon,
                       "offered_particle_steps_per_s": offered, "pool_particles": max_particles,
                       "list_skin": "adaptive" if args.list_skin is None else args.list_skin,
                       "parallelism": f"requests sharded over {world} GPU(s)"},
            "serve": got if world > 1 else summ,
            "e2e": {"value": ps / wall, "unit": "particle-steps/s",
                    "note": "every request's scene uploaded from host memory and its final state read back"},
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)


SERVE_MIX_SCENES = 64  # requests of the mix comparison (the first ones of the arrival order)
SERVE_MIX_STEPS = 20   # time steps each of them takes in both forms


def request_mix_comparison(requests, steps, device, stream):
    """Scenes of `requests` advanced `steps` time steps, once with one context per request (each context's
    step launched in turn, the plain step per scene) and once as one batch: particle-steps/s and scene-steps/s
    of both, on the same stream. The rate a served rollout mix reaches is bounded by the second form."""
    import torch

    from pcisph_gb300 import Batch, Fluid, setup_scene
    scs = [r.scene for r in requests]
    n = sum(s.fluid_count for s in scs)

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3

    ctxs = []
    for s in scs:
        f = Fluid(device, stream=stream.cuda_stream)
        setup_scene(f, s)
        f.update()  # first step (graph instantiation) untimed
        ctxs.append(f)
    t_single = timed(lambda: [f.update() for f in ctxs])
    for f in ctxs:
        f.close()
    bt = Batch(device, max_particles=n, max_scenes=len(scs), stream=stream.cuda_stream)
    for s in scs:
        bt.add_scene(s)
    bt.step(1)
    t_batch = timed(lambda: bt.step(1))
    bt.close()
    for r in requests:
        r.release()
    return {"scenes": len(scs), "particles": n, "steps": steps,
            "per_scene_contexts": {"particle_steps_per_s": n * steps / t_single,
                                   "scene_steps_per_s": len(scs) * steps / t_single},
            "batched": {"particle_steps_per_s": n * steps / t_batch, "scene_steps_per_s": len(scs) * steps / t_batch},
            "speedup_of_batch": t_single / t_batch}


def main():
    args = parse()
    rc = relaunch_as_ranks(args, sys.argv[1:])
    if rc is not None:
        sys.exit(rc)
    rank, world, local = dist_env()
    if world != args.gpus:
        sys.exit(f"bench.py: --gpus {args.gpus} but {world} rank(s) were launched")
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if args.workload in ("scenes", "serve"):
        import torch
        import torch.distributed as dist
        if world > 1:
            dist.init_process_group("gloo" if args.workload == "serve" else "nccl")
        torch.cuda.set_device(local)
        (scenes_workload if args.workload == "scenes" else serve_workload)(args, rank, world, local)
        if world > 1:
            dist.destroy_process_group()
        return
    import numpy as np
    import torch
    import torch.distributed as dist

    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from pcisph_gb300 import Fluid, build, scenes, setup_scene
    build.build()
    cfg, metric, workload = DAM_WORKLOADS[args.workload]
    sc = getattr(scenes, cfg)()
    N = sc.fluid_count
    stream = torch.cuda.Stream()  # a real stream: the library launches on it, the events are recorded on it
    torch.cuda.set_stream(stream)
    f = Fluid(local, stream=stream.cuda_stream)
    setup_scene(f, sc, kernel_variant=args.variant, loop_mode=args.loop_mode, spatial_order=args.spatial_order)
    if args.list_skin is not None:
        f.set_options(list_skin=args.list_skin)
    sampler = ClockSampler(local)
    sampler.start()
    for _ in range(args.warmup):
        f.update()
    torch.cuda.synchronize()
    tuned = f.autotune(steps=3) if args.autotune else None
    # snapshot of the state after warm-up: the profile pass, the e2e pass and the CPU baseline replay the
    # same steps as the timed loop (the step is deterministic)
    snap_pos = torch.empty((N, 4), dtype=torch.float32, device="cuda")
    snap_vel = torch.empty((N, 4), dtype=torch.float32, device="cuda")
    f.get_field("position", layout="float4", out=snap_pos)
    f.get_field("velocity", layout="float4", out=snap_vel)
    f.reset_stats()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    st0 = f.stats()
    launches0 = f.kernel_launches()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    max_err = 0.0
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        starts[k].record(stream)
        f.update()
        ends[k].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    if world > 1:
        dist.barrier()
    st1 = f.stats()
    launches = f.kernel_launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    total_ms = max_over_ranks(sum(step_ms))
    iters = (st1.total_iterations - st0.total_iterations) / max(1, st1.steps - st0.steps)
    status_bits = st1.status_all
    value = replica_value(N * args.steps, world, total_ms)

    # per-kernel CUDA events over the first steps of the timed loop again (host-driven loop, same kernels)
    prof_steps = min(args.steps, 20)
    f.set_fluid_state(snap_pos, snap_vel)
    sp0 = f.stats()
    f.profile(True)
    f.step(prof_steps)
    prof = f.profile_read()
    f.profile(False)
    sp1 = f.stats()
    prof_iters = (sp1.total_iterations - sp0.total_iterations) / max(1, sp1.steps - sp0.steps)
    clocks = sampler.stop()
    tot = sum(ms for _, ms in prof.values())
    dom = max(prof.items(), key=lambda kv: kv[1][1])
    dname, (dl, dms) = dom
    avg_s = dms / dl / 1e3
    peak, peak_kind = peaks()
    # the persistent loop (loop_mode 2) runs a step's iterations in one launch
    algo = dict(ALGO_BYTES, corrective_loop=(ALGO_BYTES["pressure"] + ALGO_BYTES["pressure_force"]) * prof_iters)
    achieved = algo.get(dname, 0) * N / avg_s / 1e9
    traffic = ncu_traffic(args.variant).get(dname)
    kernels = {k: {"launches": l, "avg_us": 1e3 * ms / l, "share": ms / tot,
                   "algo_GBps": algo.get(k, 0) * N / (ms / l / 1e3) / 1e9} for k, (l, ms) in prof.items()}

    # e2e through the C ABI with pinned host buffers, over the same steps as the timed loop
    pos_h = torch.empty((N, 3), dtype=torch.float32, pin_memory=True).numpy()
    vel_h = torch.empty((N, 3), dtype=torch.float32, pin_memory=True).numpy()
    f.set_fluid_state(snap_pos, snap_vel)
    f.get_field("position", out=pos_h)
    f.get_field("velocity", out=vel_h)
    e2e_steps = args.steps
    # the CPU baseline starts from the states at evenly spaced points of these steps (the copies are not
    # timed), so that it samples the same part of the run as the GPU's timed steps
    points = sorted({(k * e2e_steps) // CPU_POINTS for k in range(CPU_POINTS)})
    samples = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    t_copy = 0.0
    for k in range(e2e_steps):
        if k in points:
            tc = time.perf_counter()
            samples.append((pos_h.copy(), vel_h.copy()))
            t_copy += time.perf_counter() - tc
        f.set_fluid_state(pos_h, vel_h)
        f.update()
        f.get_fluid_state(pos_h, vel_h)
    e2e_s = time.perf_counter() - t0 - t_copy
    e2e = {"value": N * e2e_steps * world / e2e_s, "unit": "particle-steps/s", "h2d_bytes_per_step": 24 * N,
           "d2h_bytes_per_step": 24 * N, "steps": e2e_steps,
           "device_value_same_steps": N * e2e_steps * world / (sum(step_ms[:e2e_steps]) / 1e3),
           "host_link_GBps": host_link_rates(24 * N)}

    cand = walk_candidates(f)
    step_bytes = STEP_FIXED_BYTES + STEP_ITER_BYTES * iters
    cpu = None
    if rank == 0 and world == 1:
        rate, csteps, citers = cpu_sample_rate(sc, samples, args.cpu_seconds, max_steps=args.steps)
        cpu = {"value": rate, "unit": "particle-steps/s", "cores": oracle_threads(), "kind": "port",
               "sample": f"{N} particles x {csteps} steps, one step at a time from the states at {len(samples)} "
                         f"evenly spaced points of the timed steps (mean {citers:.2f} corrective iterations "
                         f"against the GPU's {iters:.2f}), oracle/pcisph_oracle.cpp with OpenMP",
               "mean_iterations": citers, "particle_iterations_per_s": rate * citers}
    if rank == 0:
        line = {
            "metric": metric, "value": value, "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered lattice)",
            "config": {"workload": workload, "particles": N, "parallelism": f"replicas x{world}",
                       "kernel_variant": args.variant, "loop_mode": args.loop_mode, "autotuned": tuned,
                       "mean_iterations": iters, "particle_iterations_per_s": value * iters,
                       "max_density_error_last": st1.max_density_error,
                       "list_skin": f.get_options().list_skin,
                       "list_fallback_sweeps_per_step": (st1.list_fallbacks - st0.list_fallbacks) / args.steps,
                       "fast_predictions_per_step": (st1.fast_particles - st0.fast_particles) / args.steps,
                       "step_ms_min_median_max": [min(step_ms), statistics.median(step_ms), max(step_ms)],
                       "converged_all_steps": (status_bits & 1) == 0, "status_bits": status_bits,
                       "accuracy_gate": {"threshold": sc.threshold, "steps_at_cap": int(st1.unconverged_steps),
                                         "steps": args.steps, "max_density_error": st1.max_density_error_max,
                                         "all_steps_within": int(st1.unconverged_steps) == 0},
                       "l2": "256 MB written between timed steps (not timed); step working set ~200 MB > L2",
                       "wall_s_timed_loop": wall,
                       "step_algorithmic_bytes_per_particle": step_bytes,
                       "step_hbm_frac": step_bytes * value / (peak * 1e9),
                       "walk_candidates_per_particle": cand,
                       "reference_pair_evaluations_per_s": cand * (3 + 2 * iters) * value},
            "e2e": e2e,
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": traffic * N if traffic else None,
                         "algo_bytes_per_particle": algo.get(dname, 0), "avg_launch_us": avg_s * 1e6,
                         "profile_pass_iterations_per_step": prof_iters,
                         "binding_unit": binding_unit(args.variant, dname)},
            "kernels": kernels,
            "cpu_baseline": cpu,
            "clocks": clocks,
        }
    f.close()
    if args.workload == "dam1m" and args.scenes_leg_steps > 0:
        line_b = batched_leg(args, rank, world, local)
        if rank == 0:
            line["batched_scenes"] = line_b
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def batched_leg(args, rank, world, local):
    """The batched form (256 scenes of the batched workload) over a short window, reported inside the 1M dam
    break's line: its rate, the gate and the speed-up over one context per scene. Errors are reported, not
    raised: this leg never costs the headline line."""
    import copy
    a = copy.copy(args)
    a.steps, a.warmup, a.scenes, a.list_skin, a.autotune, a.loop_mode = args.scenes_leg_steps, 3, 256, None, False, 0
    try:
        b = scenes_workload(a, rank, world, local, emit=False, cpu_leg=False)
    except Exception as e:  # noqa: BLE001 -- the leg is auxiliary
        return {"error": f"{type(e).__name__}: {e}"}
    if b is None:
        return None
    keep = ("metric", "value", "unit", "ms_per_step", "steps", "warmup", "per_scene_contexts", "e2e", "accuracy_gate",
            "gpu_launches", "clocks")
    out = {k: b[k] for k in keep if k in b}
    out["workload"] = b["config"]["workload"]
    out["mean_scene_iterations"] = b["config"]["mean_scene_iterations"]
    out["scene_steps_per_s"] = b["config"]["scene_steps_per_s"]
    return out


if __name__ == "__main__":
    main()
