"""Parameter sweeps: many variants of one scene (viscosity, surface tension, time step, gravity, rest
density, threshold) stepped together as the scenes of one batch pool (pcisph_batch_*), each with its own
parameters and convergence; every variant's result is the one it would have alone. No counterpart in the
reference, which runs one parameter set per process."""
import copy
import itertools

from .batch import Batch

SWEEPABLE = ("viscosity", "raw_viscosity", "surface_tension", "delta_t", "gravity", "rest_density", "threshold",
             "min_iters", "max_iters", "restitution")


def variants(base, **grid):
    """The cartesian product of the given parameter values applied to copies of scenes.Scene `base`, e.g.
    variants(scene, viscosity=[0.1, 0.2], delta_t=[5e-4, 1e-3]) -> 4 scenes, first parameter slowest."""
    for k in grid:
        if k not in SWEEPABLE:
            raise ValueError(f"{k} is not a sweepable parameter ({', '.join(SWEEPABLE)})")
    names = list(grid)
    out = []
    for values in itertools.product(*(grid[k] for k in names)):
        sc = copy.copy(base)
        for k, v in zip(names, values):
            setattr(sc, k, v)
        sc.name = base.name + "[" + ",".join(f"{k}={v}" for k, v in zip(names, values)) + "]"
        out.append(sc)
    return out


def run(scene_list, steps, device=0, fields=("position", "velocity"), stream=None):
    """Step every scene `steps` times in one batch; returns, per scene, a dict of the requested fields (in
    the scene's own sorted order) and its step statistics."""
    total = sum(s.fluid_count for s in scene_list)
    bt = Batch(device, max_particles=total, max_scenes=len(scene_list), stream=stream)
    try:
        ids = [bt.add_scene(s) for s in scene_list]
        bt.step(steps)
        bt.sync()
        results = []
        for sid, s in zip(ids, scene_list):
            r = {name: bt.get_field(sid, name, s.fluid_count) for name in fields}
            r["stats"] = bt.stats(sid)
            results.append(r)
        return results
    finally:
        bt.close()
