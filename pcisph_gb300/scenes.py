"""Deterministic analytic scenes for the PCISPH step.

The reference builds its scenes from ``.xraw`` voxel files
(PCISPH/src/scenes.cpp:76-149, 217-245). The workloads here are analytic
instead: jittered fluid lattices in a box with reflecting walls. Every random
number comes from a counter-based hash of (seed, particle id, axis), so a scene
is the same on every machine and in every process.

Physics maps onto the reference's parametrisation (Fluid.cpp:377-401) through
``particle_radius = d / 2``: then h = 4r = 2d and m = rho0 (2r)^3 = rho0 d^3.
"""
from dataclasses import dataclass, field

import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_GOLD = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z):
    """splitmix64 finaliser (Steele, Lea, Flood 2014), vectorised over uint64."""
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def uniform(seed, ids, axis, stream=0):
    """U[0,1) per (seed, id, axis, stream); float64 with 53 random bits."""
    with np.errstate(over="ignore"):
        ids = np.asarray(ids, np.uint64)
        base = _mix64(np.uint64(seed) * _GOLD + np.uint64(stream) * np.uint64(0xD1B54A32D192ED03))
        z = _mix64(base ^ (ids * np.uint64(4) + np.uint64(axis)) * _GOLD)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclass
class Scene:
    """One scene: initial state plus the physical parameters of the step."""
    name: str
    fluid_pos: np.ndarray                  # (N, 3) float32
    spacing: float                         # lattice spacing d
    delta_t: float
    box_lo: tuple = (0.0, 0.0, 0.0)
    box_hi: tuple = (0.0, 0.0, 0.0)
    boundary_pos: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    fluid_vel: np.ndarray = None           # (N, 3) float32 or None (zero)
    rest_density: float = 1000.0
    viscosity: float = 0.2                 # dynamic viscosity mu (Pa s)
    raw_viscosity: float = None            # the reference's viscosity_constant, if given directly
    surface_tension: float = 0.5
    gravity: float = -9.81
    threshold: float = 0.01
    min_iters: int = 3
    max_iters: int = 50
    walls: bool = True
    restitution: float = 0.5
    steps: int = 0                         # the workload's step count

    @property
    def particle_radius(self):
        return 0.5 * self.spacing

    def viscosity_constant(self):
        """The reference's viscosity_constant for dynamic viscosity mu.

        The reference's viscosity force is mu_c * m * sum_j (v_j - v_i)/rho_j * lap W
        (PCISPH/data/kernels/pcisph.cl:146, :160); Mueller et al.'s (SCA 2003) is
        (mu m / rho_i) * sum_j m (v_j - v_i)/rho_j * lap W. With rho_i = rho0 and
        m = rho0 d^3 the two agree for mu_c = mu * m / rho0 = mu * d^3. (mu = 0.2 used
        as mu_c directly makes the explicit viscosity unstable within a few steps.)
        """
        if self.raw_viscosity is not None:
            return float(self.raw_viscosity)
        return float(self.viscosity * self.spacing ** 3)

    @property
    def fluid_count(self):
        return int(self.fluid_pos.shape[0])

    @property
    def boundary_count(self):
        return int(self.boundary_pos.shape[0])


def lattice_block(nx, ny, nz, d, origin, seed, jitter=0.05, id_offset=0):
    """(nx*ny*nz, 3) float32 lattice, x fastest, points at cell centres plus U(+-jitter*d)."""
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    idx = np.stack([ix.ravel(order="F"), iy.ravel(order="F"), iz.ravel(order="F")], 1).astype(np.float64)
    n = idx.shape[0]
    ids = np.arange(n, dtype=np.uint64) + np.uint64(id_offset)
    pos = (idx + 0.5) * d + np.asarray(origin, np.float64)
    if jitter:
        for a in range(3):
            pos[:, a] += (2.0 * uniform(seed, ids, a) - 1.0) * jitter * d
    return pos.astype(np.float32)


def dam_break(n_side=32, seed=0, extent=0.64, box=(1.6, 1.2, 0.8), delta_t=None, steps=1000, **kw):
    """Dam break: an n_side^3 jittered lattice filling [0, extent]^3 in a box (1.6 x 1.2 x 0.8 m)."""
    d = extent / n_side
    if delta_t is None:
        delta_t = 1e-3 * (d / 0.02)
    pos = lattice_block(n_side, n_side, n_side, d, (0, 0, 0), seed)
    return Scene(f"dam_break_{n_side}^3", pos, d, delta_t, (0.0, 0.0, 0.0), tuple(box), steps=steps, **kw)


def dam_break_32k():
    """32,768 particles, d = 0.02 m, dt = 1e-3 s, 1000 steps."""
    return dam_break(32, seed=0, delta_t=1e-3, steps=1000)


def dam_break_1m():
    """1,048,576 particles, d = 0.005 m, dt = 2.5e-4 s, 500 steps, in the 1.6 x 1.2 x 0.8 m box.

    A 128^3 lattice at d = 0.005 m would hold 2,097,152 particles; the workload keeps the stated
    particle count (2^20) and spacing and halves the depth: 128 x 128 x 64 (0.64 x 0.64 x 0.32 m).
    """
    d = 0.005
    pos = lattice_block(128, 128, 64, d, (0.0, 0.0, 0.0), seed=0)
    return Scene("dam_break_128x128x64", pos, d, 2.5e-4, (0.0, 0.0, 0.0), (1.6, 1.2, 0.8), steps=500)


def dam_break_1m_boundary():
    """The 1,048,576-particle dam-break block (d = 0.005 m) against boundary particles: two layers of
    spacing d lining the floor and four walls of a 1.28 x 0.96 x 0.32 m box (the block fills its left half,
    the whole depth): ~290K boundary particles, the reference's boundary handling at scale (its dambreak
    scene has 154,980 boundary particles for 279,936 fluid ones). The reflecting walls stay on as well.

    With boundary particles under the fluid the column's hydrostatic pressure has to be rebuilt from zero
    every step (the reference resets pressures each step, pcisph.cl:121-173), which no iteration count
    reaches to 1% for a 0.64 m column: the workload uses the reference's own limits, 3 to 7 iterations
    (Fluid.cpp:250-251), and reports the density error it reaches."""
    d = 0.005
    pos = lattice_block(128, 128, 64, d, (0.0, 0.0, 0.0), seed=0)
    box = (1.28, 0.96, 0.32)
    b = boundary_box((0.0, 0.0, 0.0), box, d, layers=2)
    return Scene("dam_break_128x128x64_boundary", pos, d, 2.5e-4, (0.0, 0.0, 0.0), box, boundary_pos=b, steps=500,
                 min_iters=3, max_iters=7)


def two_blocks_8m():
    """8,388,608 particles: two 256x128x128 blocks (d = 0.0025 m) at opposite ends of
    [0,1.6]x[0,0.8]x[0,0.4], dt = 1.25e-4 s, 200 steps."""
    d = 0.0025
    a = lattice_block(256, 128, 128, d, (0.0, 0.0, 0.0), seed=2)
    b = lattice_block(256, 128, 128, d, (1.6 - 256 * d, 0.0, 0.0), seed=2, id_offset=256 * 128 * 128)
    pos = np.concatenate([a, b])
    return Scene("two_blocks_8M", pos, d, 1.25e-4, (0.0, 0.0, 0.0), (1.6, 0.8, 0.4), steps=200)


def small_dam(n_side=16, seed=0, **kw):
    """A small dam break with the 32K dam break's physics for tests (same spacing, fewer particles)."""
    d = 0.02
    return dam_break(n_side, seed=seed, extent=n_side * d, delta_t=1e-3, **kw)


def boundary_box(lo, hi, d, layers=2):
    """Boundary particles lining the inside of a box (floor and four side walls), reference style.

    The reference samples boundary voxels into ppd^3 particle lattices
    (scenes.cpp:88-98, 137-145); this is the analytic counterpart: ``layers``
    sheets of spacing d below the floor and outside each side wall.
    """
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    nx = int(round((hi[0] - lo[0]) / d)) + 2 * layers
    ny = int(round((hi[1] - lo[1]) / d)) + layers
    nz = int(round((hi[2] - lo[2]) / d)) + 2 * layers
    # z outermost, x fastest (the point order of the original triple loop)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x = lo[0] + (i.ravel() - layers + 0.5) * d
    y = lo[1] + (j.ravel() - layers + 0.5) * d
    z = lo[2] + (k.ravel() - layers + 0.5) * d
    inside = (lo[0] <= x) & (x <= hi[0]) & (lo[2] <= z) & (z <= hi[2]) & (y >= lo[1])
    return np.stack([x[~inside], y[~inside], z[~inside]], axis=1).astype(np.float32).reshape(-1, 3)


def _lattice_points(nx, ny, nz, d, origin):
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    idx = np.stack([ix.ravel(order="F"), iy.ravel(order="F"), iz.ravel(order="F")], 1).astype(np.float64)
    return (idx + 0.5) * d + np.asarray(origin, np.float64)


def _jitter(pos, seed, id_offset, d, jitter=0.05):
    ids = np.arange(pos.shape[0], dtype=np.uint64) + np.uint64(id_offset)
    out = pos.copy()
    for a in range(3):
        out[:, a] += (2.0 * uniform(seed, ids, a) - 1.0) * jitter * d
    return out


def batch_dam(count, aspect_x, aspect_z, d=0.01, seed=3, id_offset=0, delta_t=1e-3, name="dam"):
    """A dam-break block of about `count` particles, sides nx:ny:nz = aspect_x:1:aspect_z, in a tank
    2.5x as long and 2x as high as the block, as deep as the block."""
    ny = max(2, int(round((count / (aspect_x * aspect_z)) ** (1.0 / 3.0))))
    nx, nz = max(2, int(round(aspect_x * ny))), max(2, int(round(aspect_z * ny)))
    pos = _jitter(_lattice_points(nx, ny, nz, d, (0.0, 0.0, 0.0)), seed, id_offset, d).astype(np.float32)
    box_hi = (2.5 * nx * d, 2.0 * ny * d, nz * d)
    return Scene(name, pos, d, delta_t, (0.0, 0.0, 0.0), box_hi)


def batch_drop(count, d=0.01, seed=3, id_offset=0, delta_t=1e-3, drop_height=0.5, name="drop"):
    """A fluid sphere of 70% of `count` particles whose bottom is `drop_height` above a pool holding the
    other 30% in a square tank; the pool is half as deep as the sphere's radius, or shallower where the
    tank must be wider than the sphere."""
    n_sphere, n_pool = int(round(0.7 * count)), count - int(round(0.7 * count))
    radius = (3.0 * n_sphere / (4.0 * np.pi)) ** (1.0 / 3.0) * d
    pool_h = max(2 * d, 0.5 * radius)
    side = max(4, int(round(np.sqrt(n_pool * d / pool_h))), int(np.ceil(2.0 * radius / d)) + 2)  # sphere fits
    layers = max(1, int(round(n_pool / (side * side))))
    pool = _lattice_points(side, layers, side, d, (0.0, 0.0, 0.0))
    L = side * d
    top = layers * d
    centre = np.array([0.5 * L, top + drop_height + radius, 0.5 * L])
    m = int(np.ceil(radius / d)) + 1
    cube = _lattice_points(2 * m, 2 * m, 2 * m, d, centre - m * d)
    sphere = cube[np.linalg.norm(cube - centre, axis=1) <= radius]
    pos = np.concatenate([pool, sphere])
    pos = _jitter(pos, seed, id_offset, d).astype(np.float32)
    box_hi = (L, top + drop_height + 2.0 * radius + 2 * d, L)
    return Scene(name, pos, d, delta_t, (0.0, 0.0, 0.0), box_hi)


def batch_scenes(count=256, seed=3, n_min=4096, n_max=131072, d=0.01, delta_t=1e-3):
    """Batched scenes: `count` scenes with log-uniform particle counts in [n_min, n_max]; each a dam-break block
    (aspect ratios U[0.5, 2]) or a sphere dropped 0.5 m into a pool holding 30% of its particles."""
    out, offset = [], 0
    ids = np.arange(count, dtype=np.uint64)
    u_n = uniform(seed, ids, 0, stream=1)
    u_kind = uniform(seed, ids, 1, stream=1)
    u_ax = uniform(seed, ids, 2, stream=1)
    u_az = uniform(seed, ids, 3, stream=1)
    for k in range(count):
        n = int(round(np.exp(np.log(n_min) + u_n[k] * (np.log(n_max) - np.log(n_min)))))
        if u_kind[k] < 0.5:
            sc = batch_dam(n, 0.5 + 1.5 * u_ax[k], 0.5 + 1.5 * u_az[k], d, seed, offset, delta_t, f"dam{k}")
        else:
            sc = batch_drop(n, d, seed, offset, delta_t, name=f"drop{k}")
        offset += sc.fluid_count
        out.append(sc)
    return out
