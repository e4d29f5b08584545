"""GPU: the headless renderer (pcisph_render / pcisph_render_fluid) against a float32 numpy restatement,
and frame recording to PNG."""
import numpy as np
import pytest

from pcisph_gb300 import Fluid, render, scenes, setup_scene
from render_ref import render as render_ref

pytestmark = pytest.mark.gpu


def _agree(got, want):
    diff = np.abs(got.astype(int) - want.astype(int)).max(-1)
    assert (diff <= 2).mean() >= 0.995, f"{(diff > 2).sum()} pixels differ by more than 2"


def test_render_matches_numpy_reference():
    sc = scenes.small_dam(5, seed=3)  # 125 particles, 0.1 m
    f = Fluid(0)
    setup_scene(f, sc, kernel_variant=2)
    cam = render.camera(eye=(0.25, 0.2, 0.45), target=(0.05, 0.05, 0.05), fov_x_degrees=50.0)
    p = f.get_params()
    pos = f.get_field("position")
    got = render.render(f, cam, 96, 64)  # before any step: every particle at the neutral colour
    _agree(got, render_ref(pos, None, p.particle_radius, p.rest_density, cam, 96, 64))
    assert (got.sum(-1) > 0).mean() > 0.05
    f.step(2)
    got = render.render(f, cam, 96, 64)
    want = render_ref(f.get_field("position"), f.get_field("density"), p.particle_radius, p.rest_density, cam, 96, 64)
    _agree(got, want)
    f.close()


def test_record_writes_frames(tmp_path):
    sc = scenes.small_dam(8, seed=4)
    f = Fluid(0)
    setup_scene(f, sc, kernel_variant=2)
    cam = render.camera(eye=(0.6, 0.4, 0.9), target=(0.16, 0.08, 0.16))
    paths = render.record(f, duration=0.006, interval=0.002, out_dir=str(tmp_path), cam=cam, width=64, height=48)
    assert len(paths) == 3
    for p in paths:
        img = render.read_png(p)
        assert img.shape == (48, 64, 3) and img.max() > 0
    f.close()
