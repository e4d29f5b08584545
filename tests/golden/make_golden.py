"""Generate the golden vectors in tests/golden/ from the reference's own kernels.

The reference's OpenCL kernels (PCISPH/data/kernels/*.cl) and its parameter
derivation (PCISPH/src/sim/Fluid.cpp:377-443) are compiled on the host by
oracle/build_ref.sh; this script drives them through the reference host
sequence and stores inputs and outputs of every stage. It needs the reference
sources, so it runs only where they exist; the .npz files it writes are
committed and are what the tests read.

    python tests/golden/make_golden.py [fixture names]   (default: all)
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.reference import Reference  # noqa: E402
from pcisph_gb300 import scenes  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def params_bytes(p):
    return np.frombuffer(bytes(p), np.uint8).copy()


def gen_params(R):
    # (particle_radius, rest_density, fluid_count, boundary_count, dt, gravity, viscosity, surface_tension)
    cases = [
        (0.01, 1000.0, 32768, 0, 1e-3, -9.81, 1.6e-6, 0.5),              # 32K dam break
        (0.0025, 1000.0, 1048576, 0, 2.5e-4, -9.81, 2.5e-8, 0.5),        # 1M dam break
        (0.00125, 1000.0, 8388608, 0, 1.25e-4, -9.81, 3.125e-9, 0.5),    # 8M two blocks
        (0.5 * 0.7 / 18, 999.972, 279936, 154980, 0.002, -9.81, 8e-5, 1.0),  # reference dambreak
        (0.5 * 0.7 / 19, 999.972, 438976, 322272, 0.002, -9.81, 8e-5, 1.0),  # reference cube_splash
        (0.5 * 0.7 / 30, 999.972, 27000, 0, 0.002, 0.0, 8e-5, 1.0),          # reference simple_drop
        (0.01, 1000.0, 1, 0, 1e-3, -9.81, 0.0, 0.0),
        (0.01, 1000.0, 127, 3, 1e-3, -9.81, 0.0, 0.0),
        (0.01, 1000.0, 129, 0, 1e-3, -9.81, 0.0, 0.0),
    ]
    inputs = np.array(cases, np.float64)
    out = np.stack([params_bytes(R.derive_params(*c)) for c in cases])
    ns = np.array([1, 2, 3, 4, 5, 63, 64, 65, 1000, 32768, 1048575, 1048576, 1048577, 8388608, 2**31, 2**32 - 1],
                  np.uint64)
    np.savez_compressed(os.path.join(OUT, "params.npz"), inputs=inputs, params=out, sort_bits_n=ns)


def gen_hash(R):
    """Keys of adversarial positions: cell borders, +-1 ulp, negatives, saturation, NaN, inf."""
    rng = np.random.default_rng(11)
    cell = np.float32(0.04)
    base = np.array([0.0, -0.0, 0.04, -0.04, 0.08, 0.12, 1.0, -1.0, 0.64, 1e-30, -1e-30, 123.456, -987.25,
                     8.5e7, -8.5e7, 3e9, -3e9, 1e20, -1e20, np.inf, -np.inf, np.nan], np.float32)
    near = []
    for k in range(-6, 7):
        v = np.float32(k) * cell
        near += [v, np.nextafter(v, np.float32(np.inf)), np.nextafter(v, np.float32(-np.inf))]
    vals = np.concatenate([base, np.array(near, np.float32)])
    combos = rng.choice(vals, size=(1500, 3)).astype(np.float32)
    rand = (rng.standard_normal((1000, 3)) * 2.0).astype(np.float32)
    big = (rng.uniform(-1, 1, (500, 3)) * 2.0e8).astype(np.float32)
    pos = np.concatenate([combos, rand, big]).astype(np.float32)
    out = {"pos": pos}
    from oracle.oracle import SimParams
    for bk in (64, 16384, 524288, 4194304, 64 * 999983):
        p = SimParams()
        p.cell_size = cell
        p.bucket_count = bk
        keys, _ = R.initialize(p, pos)
        out[f"keys_{bk}"] = keys
    np.savez_compressed(os.path.join(OUT, "hash.npz"), cell=np.float32(cell), **out)


def gen_sort(R):
    rng = np.random.default_rng(12)
    out = {}
    for i, (n, hi) in enumerate([(1, 10), (63, 5), (64, 64), (65, 1 << 20), (1000, 3), (2049, 1 << 19),
                                 (3000, 1 << 31)]):
        keys = rng.integers(0, hi, n, dtype=np.uint64).astype(np.uint32)
        vals = np.arange(n, dtype=np.uint32)
        sk, sv = R.stable_sort(keys, vals)
        out[f"keys_{i}"], out[f"sorted_keys_{i}"], out[f"sorted_vals_{i}"] = keys, sk, sv
    np.savez_compressed(os.path.join(OUT, "sort.npz"), **out)


def chain(R, p, f_pos0, f_vel0, b_pos0):
    """Every kernel once in reference order, recording inputs and outputs."""
    g = {"params": params_bytes(p), "f_pos0": f_pos0, "f_vel0": f_vel0, "b_pos0": b_pos0}
    N, B, bk = p.fluid_count, p.boundary_count, p.bucket_count
    if B:
        bk_, bs_ = R.initialize(p, b_pos0)
        bk_, bs_ = R.stable_sort(bk_, bs_)
        b_pos, b_off = R.reorder_boundary(p, bk_, bs_, b_pos0)
        g.update(b_keys=bk_, b_src=bs_, b_pos=b_pos, b_off=b_off)
        g["b_init"] = R.boundary_self_density(p, b_off, b_pos)
    else:
        b_pos, b_off = np.zeros((0, 3), np.float32), np.zeros(2 * bk, np.uint32)
    keys, src = R.initialize(p, f_pos0)
    g["f_keys_unsorted"] = keys
    keys, src = R.stable_sort(keys, src)
    f_pos, f_vel, f_off = R.reorder_fluid(p, keys, src, f_pos0, f_vel0)
    g.update(f_keys=keys, f_src=src, f_pos=f_pos, f_vel=f_vel, f_off=f_off)
    rho = R.update_density(p, b_off, b_pos, f_off, f_pos)
    nrm = R.update_normal(p, f_off, f_pos, rho)
    fo, pr, fp = R.force_init(p, f_off, f_pos, nrm, rho, f_vel)
    g.update(rho=rho, normal=nrm, f_other=fo)
    b_init0 = np.zeros(B, np.float32)
    b_press = np.zeros(B, np.float32)
    for it in range(2):
        pred = R.advance(p, f_pos, f_vel, fo, fp, integrate=False)
        if B:
            b_press, _ = R.update_pressure(p, 1, b_off, b_pos, b_init0, f_off, f_pos, pred, b_press)
            bpc, _ = R.update_pressure(p, 1, b_off, b_pos, g["b_init"], f_off, f_pos, pred,
                                       np.zeros(B, np.float32))
            g[f"b_press_computed{it}_from0"] = bpc
        pr_in = pr.copy()
        pr, err = R.update_pressure(p, 0, b_off, b_pos, b_init0, f_off, f_pos, pred, pr)
        fp = R.pressure_force(p, b_off, b_pos, b_press, f_off, f_pos, rho, pr)
        g.update({f"pred{it}": pred, f"press_in{it}": pr_in, f"press{it}": pr, f"err{it}": err, f"fpress{it}": fp,
                  f"b_press{it}": b_press.copy()})
    x1, v1 = R.advance(p, f_pos, f_vel, fo, fp, integrate=True)
    g.update(x_new=x1, v_new=v1)
    return g


def full_steps(R, p, f_pos0, f_vel0, b_pos0, nsteps, max_iters=7, threshold=0.01):
    from oracle.oracle import get
    s = get().new_state(p, f_pos0, f_vel0, b_pos0)
    out = {}
    for k in range(nsteps):
        it, me = R.step(p, threshold, max_iters, k == 0, 0, s)
        out[f"step{k}_iters"] = np.int32(it)
        out[f"step{k}_max_err"] = np.float32(me)
        for n in ("f_pos", "f_vel", "f_normal", "f_pred", "f_rho", "f_other", "f_press", "f_fpress", "f_err",
                  "f_src", "b_press"):
            out[f"step{k}_{n}"] = s[n].copy()
    out["b_pos_sorted"] = s["b_pos"].copy()
    return out


def gen_scene(R, name, sc, b_pos0, viscosity, surface_tension, gravity, rest_density, vel_scale, nsteps, seed):
    N, B = sc.fluid_count, b_pos0.shape[0]
    p = R.derive_params(sc.particle_radius, rest_density, N, B, sc.delta_t, gravity, viscosity, surface_tension)
    rng = np.random.default_rng(seed)
    f_vel0 = (rng.standard_normal((N, 3)) * vel_scale).astype(np.float32)
    g = chain(R, p, sc.fluid_pos, f_vel0, b_pos0)
    g.update(full_steps(R, p, sc.fluid_pos, f_vel0, b_pos0, nsteps))
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **g)
    print(name, "N", N, "B", B, "iters", [int(g[f"step{k}_iters"]) for k in range(nsteps)])


XRAW_SCENES = ("simple_drop", "dambreak", "cube_splash")


def gen_xraw():
    """The reference's three voxel scenes (PCISPH/data/scenes/*.xraw) as voxel grids, with what the
    reference's own loader (scenes.cpp:76-149) makes of them at its particles-per-voxel settings
    (scenes.cpp:229-236) and at 3: particle counts and SHA-256 of the float32 position arrays."""
    import hashlib
    import struct

    from oracle.build import REFERENCE_ROOT
    from oracle.reference import load_xraw_reference
    from pcisph_gb300.xraw import REFERENCE_SCENES
    out = {}
    for name in XRAW_SCENES:
        path = os.path.join(REFERENCE_ROOT, "PCISPH", "data", "scenes", name + ".xraw")
        data = open(path, "rb").read()
        sx, sy, sz, _ = struct.unpack_from("<4I", data, 8)
        out[f"{name}_size"] = np.array([sx, sy, sz], np.uint32)
        out[f"{name}_voxels"] = np.frombuffer(data, np.uint8, count=sx * sy * sz, offset=24).reshape(sz, sy, sx).copy()
        for ppd in sorted({REFERENCE_SCENES[name]["particles_per_dimension"], 3}):
            arrays = load_xraw_reference(path, ppd, 0.7)
            for kind, a in zip(("fluid", "boundary", "cubes"), arrays):
                out[f"{name}_ppd{ppd}_{kind}_count"] = np.int64(a.shape[0])
                out[f"{name}_ppd{ppd}_{kind}_sha256"] = np.array(hashlib.sha256(a.tobytes()).hexdigest())
        print(name, (sx, sy, sz), {k: int(v) for k, v in out.items() if k.startswith(name) and k.endswith("count")})
    np.savez_compressed(os.path.join(OUT, "xraw_scenes.npz"), **out)


def gen_dambreak_steps(R):
    """The reference's dambreak scene (decoded by its own loader at 3 particles per voxel edge, boundary
    particles included) stepped by the reference's own kernels with its settings (scenes.cpp:219-224)."""
    from oracle.build import REFERENCE_ROOT
    from oracle.reference import load_xraw_reference
    path = os.path.join(REFERENCE_ROOT, "PCISPH", "data", "scenes", "dambreak.xraw")
    fluid, boundary, _ = load_xraw_reference(path, 3, 0.7)
    sc = scenes.Scene("dambreak_ppd3", fluid, 0.7 / 3, 0.002, walls=False)
    gen_scene(R, "step_dambreak", sc, boundary, 8e-5, 1.0, -9.81, 999.972, 0.0, 3, seed=9)


GENERATORS = {
    "params": lambda R: gen_params(R), "hash": lambda R: gen_hash(R), "sort": lambda R: gen_sort(R),
    "step_boundary": None, "step_fluid": None, "xraw_scenes": lambda R: gen_xraw(),
    "step_dambreak": lambda R: gen_dambreak_steps(R),
}


def main(names):
    R = Reference()
    names = names or list(GENERATORS)
    for name in names:
        if name == "step_boundary":
            # reference-style scene: fluid block in a box lined with boundary particles (reference defaults,
            # scenes.cpp:219-224, with the dambreak resolution ppd = 18 at scaling 0.7)
            d = 0.7 / 18
            sc = scenes.dam_break(9, seed=5, extent=9 * d, box=(0, 0, 0), delta_t=0.002)
            b_pos0 = scenes.boundary_box((0, 0, 0), (12 * d, 12 * d, 12 * d), d, layers=1)
            gen_scene(R, "step_boundary", sc, b_pos0, 8e-5, 1.0, -9.81, 999.972, 0.05, 2, seed=6)
        elif name == "step_fluid":
            # fluid only, the 32K dam break's physics (no walls in the reference)
            sc = scenes.small_dam(10, seed=7)
            gen_scene(R, "step_fluid", sc, np.zeros((0, 3), np.float32), 1.6e-6, 0.5, -9.81, 1000.0, 0.05, 2,
                      seed=8)
        else:
            GENERATORS[name](R)


if __name__ == "__main__":
    main(sys.argv[1:])
