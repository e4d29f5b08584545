"""CPU: the .xraw scene loader (pcisph_gb300/xraw.py) against the reference's own loader
(PCISPH/src/scenes.cpp:76-149): the golden fixture holds the reference's three voxel scenes and what the
reference loader made of them (counts and SHA-256 of the position arrays)."""
import hashlib
import os

import numpy as np
import pytest

from pcisph_gb300 import xraw

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "xraw_scenes.npz")
SCENES = ("simple_drop", "dambreak", "cube_splash")


def _grid(g, name):
    return xraw.VoxelGrid(tuple(int(v) for v in g[f"{name}_size"]), g[f"{name}_voxels"])


@pytest.mark.parametrize("name", SCENES)
def test_loader_matches_reference_loader(name):
    g = np.load(GOLDEN)
    grid = _grid(g, name)
    for ppd in sorted({xraw.REFERENCE_SCENES[name]["particles_per_dimension"], 3}):
        got = xraw.load(grid, ppd, 0.7)
        for kind, a in zip(("fluid", "boundary", "cubes"), got):
            assert a.dtype == np.float32 and a.shape[1] == 3
            assert a.shape[0] == int(g[f"{name}_ppd{ppd}_{kind}_count"]), (name, ppd, kind)
            assert hashlib.sha256(a.tobytes()).hexdigest() == str(g[f"{name}_ppd{ppd}_{kind}_sha256"]), (name, ppd, kind)


def test_known_scene_sizes():
    """Particle counts of the reference scenes at their own resolutions."""
    g = np.load(GOLDEN)
    want = {"dambreak": (279936, 154980), "cube_splash": (438976, 322272), "simple_drop": (27000, 0)}
    for name, (nf, nb) in want.items():
        ppd = xraw.REFERENCE_SCENES[name]["particles_per_dimension"]
        assert (int(g[f"{name}_ppd{ppd}_fluid_count"]), int(g[f"{name}_ppd{ppd}_boundary_count"])) == (nf, nb)


def test_encode_parse_round_trip_and_blockers():
    vox = np.zeros((2, 3, 4), np.uint8)          # z, y, x
    vox[0, 0, 0] = xraw.FLUID
    vox[0, 0, 1] = xraw.BLOCKER                  # +x neighbour of the fluid voxel: cut to 3 layers
    vox[1, 2, 3] = xraw.BOUNDARY_INVISIBLE
    vox[0, 2, 0] = xraw.BOUNDARY_VISIBLE
    grid = xraw.VoxelGrid((4, 3, 2), vox)
    back = xraw.parse(xraw.encode(grid))
    assert back.size == grid.size and np.array_equal(back.voxels, vox)
    fluid, boundary, cubes = xraw.load(grid, 5, 1.0)
    assert fluid.shape[0] == 3 * 5 * 5              # x layers 0..2 of 5
    assert boundary.shape[0] == 2 * 125 and cubes.shape[0] == 1
    # x, z, y axis order and centring (scenes.cpp:81-85)
    ps = np.float32(1.0) / np.float32(5)
    assert fluid[:, 0].max() == np.float32(2) * ps + np.float32(-0.5 * 4)
    assert fluid[:, 1].max() == np.float32(4) * ps + np.float32(-0.5 * 2)   # file z -> position y
    with pytest.raises(ValueError):
        xraw.parse(b"NOPE" + bytes(40))


def test_reference_scene_settings():
    g = np.load(GOLDEN)
    sc = xraw.reference_scene(_grid(g, "dambreak"), "dambreak", particles_per_dimension=3)
    assert sc.fluid_count == 1296 and sc.boundary_count == 5400
    assert sc.particle_radius == pytest.approx(0.5 * 0.7 / 3)
    assert sc.delta_t == 0.002 and sc.viscosity_constant() == pytest.approx(8e-5) and not sc.walls
    drop = xraw.reference_scene(_grid(g, "simple_drop"), "simple_drop")
    assert drop.fluid_count == 27000 and drop.gravity == 0.0
