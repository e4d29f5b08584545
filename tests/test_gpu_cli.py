"""GPU: the headless C++ runner (the reference's main loop without a window) on the reference's dambreak
scene gives the same final state as the Python path through the same C ABI."""
import os
import subprocess

import numpy as np
import pytest

from pcisph_gb300 import Fluid, build, render, setup_scene, xraw

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "xraw_scenes.npz")


def test_runner_matches_python_path(tmp_path):
    g = np.load(GOLDEN)
    grid = xraw.VoxelGrid(tuple(int(v) for v in g["dambreak_size"]), g["dambreak_voxels"])
    path = tmp_path / "dambreak.xraw"
    path.write_bytes(xraw.encode(grid))
    dump = tmp_path / "pos.bin"
    frames = tmp_path / "frames"
    frames.mkdir()
    r = subprocess.run([build.build_cli(), "-i", str(path), "--ppd", "3", "--steps", "4", "--dump", str(dump),
                        "--frames", str(frames), "--every", "0.004", "--size", "64x48"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "Fluid-Particles: 1296" in r.stdout and "Boundary-Particles: 5400" in r.stdout
    got = np.fromfile(dump, np.float32).reshape(-1, 3)
    sc = xraw.reference_scene(grid, "dambreak", particles_per_dimension=3)
    f = Fluid(0)
    setup_scene(f, sc, walls=False, max_iters=7, min_iters=3)
    f.step(4)
    np.testing.assert_array_equal(got, f.get_field("position"))
    f.close()
    ppm = sorted(frames.iterdir())
    assert len(ppm) == 2
    data = ppm[0].read_bytes()
    assert data.startswith(b"P6\n64 48\n255\n") and len(data) == len(b"P6\n64 48\n255\n") + 64 * 48 * 3
