"""CPU: the synthetic workloads (sizes, determinism) and the batch memory model."""
import numpy as np

from pcisph_gb300 import scenes
from pcisph_gb300.batch import memory_model


def test_batch_scenes_shape_and_determinism():
    a = scenes.batch_scenes(count=64, seed=3)
    b = scenes.batch_scenes(count=64, seed=3)
    n = np.array([s.fluid_count for s in a])
    assert len(a) == 64
    assert n.min() >= 0.85 * 4096 and n.max() <= 1.1 * 131072
    assert {s.name[:3] for s in a} == {"dam", "dro"}
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x.fluid_pos, y.fluid_pos)
    for s in a:  # every particle starts inside its tank
        assert (s.fluid_pos >= np.asarray(s.box_lo) - s.spacing).all()
        assert (s.fluid_pos <= np.asarray(s.box_hi) + s.spacing).all()


def test_drop_scene_has_pool_and_sphere():
    s = scenes.batch_drop(20000, d=0.01, seed=1)
    y = s.fluid_pos[:, 1]
    pool_top = np.sort(y)[int(0.3 * s.fluid_count) - 1]
    gap = y[y > pool_top + 0.02]
    assert 0.6 * s.fluid_count <= gap.size <= 0.72 * s.fluid_count
    assert gap.min() - pool_top > 0.45  # dropped from 0.5 m above the pool


def test_batch_memory_model():
    per_particle, per_scene = memory_model()
    # 11 float4 state and work arrays, scalars, 168 skin-list and 64 within-h list entries, buckets, sort
    assert per_particle == 11 * 16 + 3 * 4 + 4 * 4 + 2 + (168 + 64) * 4 + 5 + 12 and per_scene > 0


def test_parameter_sweep_variants_are_a_product():
    from pcisph_gb300 import param_sweep
    base = scenes.small_dam(4)
    vs = param_sweep.variants(base, viscosity=[0.1, 0.2, 0.3], surface_tension=[0.5, 1.0])
    assert [(v.viscosity, v.surface_tension) for v in vs] == [(a, b) for a in (0.1, 0.2, 0.3) for b in (0.5, 1.0)]
    assert base.viscosity == 0.2 and all(v.fluid_pos is base.fluid_pos for v in vs)
    import pytest
    with pytest.raises(ValueError):
        param_sweep.variants(base, colour=[1])
