"""Headless scene ingest: the reference's .xraw voxel scenes as particle sets.

Restates PCISPH/src/scenes.cpp:13-149 (xraw::Data, load_xraw_host) and the scene settings of
scene::load (scenes.cpp:217-245) without OpenGL: a voxel of type fluid becomes a ppd^3 block of fluid
particles, a boundary voxel (visible or invisible) a block of boundary particles, and a block next to a
"blocker" voxel is cut to 3 particle layers on that side. Positions are (x, z, y) of the voxel grid (the
file's z axis is up), scaled and centred as the reference does, in float32 with the reference's operation
order. The file format is XRAW: a 24-byte header (magic "XRAW", channel data type, channel count, bits per
channel, bits per index, volume size x/y/z as uint32, palette colour count) followed by one byte per voxel,
x fastest.
"""
import struct
from dataclasses import dataclass

import numpy as np

BOUNDARY_VISIBLE, BOUNDARY_INVISIBLE, BLOCKER, FLUID = 1, 2, 3, 4

# scene::load (scenes.cpp:217-240): particles per voxel edge and gravity per scene; the rest is shared
REFERENCE_SCENES = {
    "simple_drop": {"particles_per_dimension": 30, "gravity": 0.0},
    "cube_splash": {"particles_per_dimension": 19, "gravity": -9.81},
    "dambreak": {"particles_per_dimension": 18, "gravity": -9.81},
}
REFERENCE_SETTINGS = {"delta_t": 0.002, "rest_density": 999.972, "viscosity": 0.00008, "surface_tension": 1.0,
                      "threshold": 0.01, "scaling": 0.7}


@dataclass
class VoxelGrid:
    size: tuple          # (x, y, z)
    voxels: np.ndarray   # uint8, shape (z, y, x)

    def type_at(self, x, y, z):
        """Voxel values at integer coordinates (arrays); outside the grid: 0 (empty)."""
        sx, sy, sz = self.size
        x, y, z = np.asarray(x, np.int64), np.asarray(y, np.int64), np.asarray(z, np.int64)
        inside = (x >= 0) & (x < sx) & (y >= 0) & (y < sy) & (z >= 0) & (z < sz)
        out = np.zeros(np.broadcast(x, y, z).shape, np.uint8)
        out[inside] = self.voxels[z[inside], y[inside], x[inside]]
        return out


def parse(data):
    """A VoxelGrid from the bytes of an .xraw file."""
    if len(data) < 24 or data[:4] != b"XRAW":
        raise ValueError("not an XRAW file")
    sx, sy, sz, _palette = struct.unpack_from("<4I", data, 8)
    n = sx * sy * sz
    if len(data) < 24 + n:
        raise ValueError("XRAW file shorter than its volume")
    vox = np.frombuffer(data, np.uint8, count=n, offset=24).reshape(sz, sy, sx).copy()
    return VoxelGrid((sx, sy, sz), vox)


def encode(grid, palette_colors=256):
    """The bytes of an .xraw file holding grid (8-bit indices; the palette is left zero)."""
    sx, sy, sz = grid.size
    head = b"XRAW" + bytes([0, 4, 8, 8]) + struct.pack("<4I", sx, sy, sz, palette_colors)
    return head + np.ascontiguousarray(grid.voxels, np.uint8).tobytes() + bytes(4 * palette_colors)


def load(grid, particles_per_dimension, scaling):
    """(fluid positions, boundary positions, visible boundary cube positions), each (n, 3) float32, in the
    reference's order (scenes.cpp:76-149)."""
    ppd = int(particles_per_dimension)
    f32 = np.float32
    ps = f32(scaling) / f32(ppd)
    sx, sy, sz = grid.size
    off = (f32(-0.5) * f32(scaling) * f32(sx), f32(-0.5) * f32(scaling) * f32(sz), f32(-0.5) * f32(scaling) * f32(sy))
    fluid, boundary, cubes = [], [], []
    for z in range(sz):
        for y in range(sy):
            for x in range(sx):
                t = int(grid.voxels[z, y, x])
                if t == BOUNDARY_VISIBLE:
                    cubes.append((f32(x) * f32(scaling) + off[0], f32(z) * f32(scaling) + off[1],
                                  f32(y) * f32(scaling) + off[2]))
                if t not in (BOUNDARY_VISIBLE, BOUNDARY_INVISIBLE, FLUID):
                    continue
                lo = [x * ppd, y * ppd, z * ppd]
                hi = [lo[0] + ppd - 1, lo[1] + ppd - 1, lo[2] + ppd - 1]
                for a, (dx, dy, dz) in enumerate(((1, 0, 0), (0, 1, 0), (0, 0, 1))):
                    c = (x, y, z)[a]
                    if int(grid.type_at(x + dx, y + dy, z + dz)) == BLOCKER:
                        hi[a] = c * ppd + 2
                    if int(grid.type_at(x - dx, y - dy, z - dz)) == BLOCKER:
                        lo[a] = (c + 1) * ppd - 3
                if hi[0] < lo[0] or hi[1] < lo[1] or hi[2] < lo[2]:
                    continue
                kz, ky, kx = np.meshgrid(np.arange(lo[2], hi[2] + 1), np.arange(lo[1], hi[1] + 1),
                                         np.arange(lo[0], hi[0] + 1), indexing="ij")
                block = np.stack([kx.ravel().astype(f32) * ps + off[0], kz.ravel().astype(f32) * ps + off[1],
                                  ky.ravel().astype(f32) * ps + off[2]], axis=1)
                (fluid if t == FLUID else boundary).append(block)
    stack = lambda parts: np.concatenate(parts).astype(f32) if parts else np.zeros((0, 3), f32)
    return stack(fluid), stack(boundary), np.array(cubes, f32).reshape(-1, 3)


def reference_scene(grid, name, particles_per_dimension=None):
    """A scenes.Scene with the reference's settings for scene `name` (scenes.cpp:217-245): dt 0.002 s,
    rest density 999.972, viscosity constant 0.00008, surface tension 1, threshold 1%, scaling 0.7, the
    scene's particles per voxel edge (or the given one) and gravity; no walls, 3..7 iterations."""
    from .scenes import Scene
    cfg = REFERENCE_SCENES[name]
    ppd = particles_per_dimension or cfg["particles_per_dimension"]
    s = REFERENCE_SETTINGS
    fluid, boundary, _ = load(grid, ppd, s["scaling"])
    spacing = s["scaling"] / ppd  # particle radius = 0.5 * scaling / ppd (scenes.cpp:166)
    return Scene(name, fluid, spacing, s["delta_t"], boundary_pos=boundary, rest_density=s["rest_density"],
                 raw_viscosity=s["viscosity"], surface_tension=s["surface_tension"], gravity=cfg["gravity"],
                 threshold=s["threshold"], min_iters=3, max_iters=7, walls=False)
