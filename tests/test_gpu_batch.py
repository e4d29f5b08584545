"""GPU: the batched multi-scene step (pcisph_batch_* C ABI) against the same scenes stepped alone.

A scene in a batch sorts into its own bucket range of the shared cell table, keeps its relative particle
order (the radix sort is stable), and walks the same neighbours in the same order with its own parameters;
its loop decision uses its own threshold and limits. Its result must therefore be the result of the same
scene in its own context, bit for bit: positions, velocities, densities and the iteration counts.
"""
import numpy as np
import pytest

from pcisph_gb300 import Batch, Fluid, scenes, setup_scene
from pcisph_gb300._lib import PcisphError

pytestmark = pytest.mark.gpu

FIELDS = ("position", "velocity", "density", "pressure")


def _mixed_scenes():
    """Scenes of different sizes, shapes, spacings and loop settings."""
    a = scenes.small_dam(8, seed=1)
    b = scenes.small_dam(11, seed=2)
    b.min_iters = b.max_iters = 4            # fixed iteration count
    c = scenes.batch_dam(3000, 1.6, 0.7, d=0.01, seed=4)
    c.threshold = 0.002                      # tighter: more iterations than the others
    d = scenes.batch_drop(5000, d=0.01, seed=5)  # falls 0.5 m: fast particles near the pool
    e = scenes.batch_dam(700, 0.6, 1.8, d=0.01, seed=6)
    e.walls = False
    return [a, b, c, d, e]


def _alone(sc, steps):
    f = Fluid(0)
    setup_scene(f, sc, kernel_variant=2)
    f.step(steps)
    out = {n: f.get_field(n) for n in FIELDS}
    st = f.stats()
    return out, (st.iterations, st.steps, st.total_iterations, st.status_all)


def _in_batch(bt, sid, sc):
    out = {n: bt.get_field(sid, n, sc.fluid_count) for n in FIELDS}
    st = bt.stats(sid)
    return out, (st.iterations, st.steps, st.total_iterations, st.status_all)


def _assert_same(name, got, want):
    for n in FIELDS:
        np.testing.assert_array_equal(got[0][n], want[0][n], err_msg=f"{name}: {n}")
    assert got[1] == want[1], (name, got[1], want[1])


def test_batch_scenes_match_alone():
    sc = _mixed_scenes()
    steps = 12
    bt = Batch(0, max_particles=sum(s.fluid_count for s in sc) + 100, max_scenes=8)
    ids = [bt.add_scene(s) for s in sc]
    assert bt.info()[:2] == (len(sc), sum(s.fluid_count for s in sc))
    bt.step(steps)
    bt.sync()
    iters = set()
    for s, sid in zip(sc, ids):
        got = _in_batch(bt, sid, s)
        want = _alone(s, steps)
        _assert_same(s.name, got, want)
        iters.add(got[1][2])
    assert len(iters) > 1  # the scenes did iterate differently
    assert bt.kernel_launches() > 0


def test_batch_remove_and_add_scenes():
    sc = _mixed_scenes()
    bt = Batch(0, max_particles=sum(s.fluid_count for s in sc), max_scenes=len(sc))
    ids = [bt.add_scene(s) for s in sc[:4]]
    bt.step(5)
    bt.remove_scene(ids[1])  # compacts the later scenes and moves their statistics
    with pytest.raises(PcisphError):
        bt.stats(ids[1])
    e_id = bt.add_scene(sc[4])
    bt.step(4)
    bt.sync()
    for k in (0, 2, 3):
        _assert_same(sc[k].name, _in_batch(bt, ids[k], sc[k]), _alone(sc[k], 9))
    _assert_same(sc[4].name, _in_batch(bt, e_id, sc[4]), _alone(sc[4], 4))
    assert bt.info()[0] == 4
    inst, upd = bt.graph_stats()
    assert inst == 1 and upd == 1  # the change of composition updated the step graph in place


def test_batch_limits_and_errors():
    a = scenes.small_dam(6, seed=1)
    bt = Batch(0, max_particles=a.fluid_count * 2, max_scenes=2)
    bt.step(1)  # empty batch: no-op
    s0 = bt.add_scene(a)
    bt.add_scene(a)
    with pytest.raises(PcisphError):
        bt.add_scene(a)  # no scene slot left
    with pytest.raises(PcisphError):
        bt.remove_scene(12345)
    with pytest.raises(PcisphError):
        bt.get_field(s0, "keys", a.fluid_count)
    bt.remove_scene(s0)
    big = scenes.small_dam(7, seed=1)
    with pytest.raises(PcisphError):
        bt.add_scene(big)  # more particles than are free
    bt.step(2)
    bt.sync()
    assert bt.info()[:2] == (1, a.fluid_count)


def test_batch_of_identical_scenes_is_identical():
    a = scenes.batch_drop(3000, d=0.01, seed=8)
    bt = Batch(0, max_particles=4 * a.fluid_count, max_scenes=4)
    ids = [bt.add_scene(a) for _ in range(4)]
    bt.step(6)
    bt.sync()
    first = _in_batch(bt, ids[0], a)
    for sid in ids[1:]:
        _assert_same("copy", _in_batch(bt, sid, a), first)


def test_parameter_sweep_variants_match_alone():
    from pcisph_gb300 import param_sweep
    base = scenes.batch_dam(1500, 1.2, 0.8, d=0.01, seed=14)
    vs = param_sweep.variants(base, viscosity=[0.1, 0.4], delta_t=[5e-4, 1e-3])
    assert len(vs) == 4 and len({(v.viscosity, v.delta_t) for v in vs}) == 4
    res = param_sweep.run(vs, steps=6, fields=FIELDS)
    for v, r in zip(vs, res):
        want = _alone(v, 6)
        _assert_same(v.name, (r, (r["stats"].iterations, r["stats"].steps, r["stats"].total_iterations,
                                  r["stats"].status_all)), want)


def test_persistent_loop_batch_matches_graph_loop():
    """loop_mode 2 runs the corrective loop as one cooperative kernel with per-scene flags: same bits as
    the graph's WHILE node, scene by scene."""
    sc = _mixed_scenes()
    out = []
    for mode in (0, 2):
        bt = Batch(0, max_particles=sum(s.fluid_count for s in sc), max_scenes=len(sc), loop_mode=mode)
        ids = [bt.add_scene(s) for s in sc]
        bt.step(8)
        bt.sync()
        out.append([_in_batch(bt, i, s) for i, s in zip(ids, sc)])
        bt.close()
    for s, a, b in zip(sc, out[0], out[1]):
        _assert_same(s.name, b, a)


def test_batch_autotune_leaves_results_unchanged():
    sc = _mixed_scenes()
    out = []
    for tune in (False, True):
        bt = Batch(0, max_particles=sum(s.fluid_count for s in sc), max_scenes=len(sc))
        ids = [bt.add_scene(s) for s in sc]
        bt.step(2)
        if tune:
            r = bt.autotune(steps=1)
            assert r["candidates"] == 24 and r["ms_per_step"] <= r["ms_per_step_before"]
        bt.step(4)
        bt.sync()
        out.append([_in_batch(bt, i, s) for i, s in zip(ids, sc)])
        bt.close()
    for s, a, b in zip(sc, out[0], out[1]):
        _assert_same(s.name, b, a)


def test_batch_bounded_sync():
    from pcisph_gb300._lib import ERR_TIMEOUT
    a = scenes.small_dam(40, seed=3)
    bt = Batch(0, max_particles=2 * a.fluid_count, max_scenes=2)
    ids = [bt.add_scene(a) for _ in range(2)]
    bt.step(1)
    bt.sync()
    bt.step(100)
    with pytest.raises(PcisphError) as e:
        bt.sync(timeout_ms=0)
    assert e.value.code == ERR_TIMEOUT
    bt.sync(timeout_ms=600000)
    assert all(bt.stats(i).steps == 101 for i in ids)


@pytest.mark.parametrize("mode", [0, 2])
def test_profiled_batch_steps_match_graph_steps(mode):
    """Profiled batch steps (host-driven, every launch timed) compute the graph's bits and time every kernel."""
    sc = _mixed_scenes()
    out = []
    for prof in (False, True):
        bt = Batch(0, max_particles=sum(s.fluid_count for s in sc), max_scenes=len(sc), loop_mode=mode)
        ids = [bt.add_scene(s) for s in sc]
        bt.step(2)
        if prof:
            bt.profile(True)
        bt.step(4)
        bt.sync()
        if prof:
            t = bt.profile_read()
            bt.profile(False)
            want = {"hash", "radix_sort", "reorder", "density", "normal", "force"} | (
                {"corrective_loop"} if mode == 2 else {"pressure", "decide", "pressure_force"})
            assert want <= set(t), t
            assert t["density"][0] == 4 and all(ms > 0 for _, ms in t.values())
        out.append([_in_batch(bt, i, s) for i, s in zip(ids, sc)])
        bt.close()
    for s, a, b in zip(sc, out[0], out[1]):
        _assert_same(s.name, b, a)


def test_adaptive_skin_follows_the_displacements_and_changes_no_bits():
    """A block thrown along the floor at 6 m/s moves 0.15 h per prediction (h = 0.04 m, dt = 1 ms), past
    half of the 0.25 h skin: with the adaptive skin its scene widens its lists (0.35 h) while a scene at
    rest keeps 0.25 h; every skin, fixed or adaptive, computes the same bits."""
    thrown = scenes.small_dam(9, seed=21)
    rest = scenes.small_dam(7, seed=22)
    v_thrown = np.zeros_like(thrown.fluid_pos)
    v_thrown[:, 0] = 6.0
    out, skins = {}, []
    for skin in ("adaptive", 0.25, 0.5):
        bt = Batch(0, max_particles=thrown.fluid_count + rest.fluid_count, max_scenes=2)
        bt.set_list_skin(skin)
        a = bt.add_scene(thrown, vel=v_thrown)
        b = bt.add_scene(rest)
        for _ in range(8):
            bt.step(5)
            if skin == "adaptive":
                skins.append((bt.stats(a).list_skin, bt.stats(b).list_skin))
        bt.sync()
        out[skin] = [_in_batch(bt, a, thrown), _in_batch(bt, b, rest)]
        bt.close()
    for skin in (0.25, 0.5):
        _assert_same("thrown", out[skin][0], out["adaptive"][0])
        _assert_same("rest", out[skin][1], out["adaptive"][1])
    assert skins[0][0] > 0.25, skins
    assert all(abs(r - 0.25) < 1e-6 for _, r in skins), skins
