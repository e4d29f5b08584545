"""CPU: the oracle against the reference's own kernels (compiled on the host by oracle/build_ref.sh) on
randomised inputs, beyond the committed golden vectors: keys, the stable permutation and cell ranges for
positions drawn across cell borders and negative coordinates, and whole Fluid::update steps of random
scenes (with and without boundary particles, random physical parameters), all bit for bit. Runs where
the reference sources exist; skipped elsewhere."""
import numpy as np
import pytest

from oracle.oracle import make_options

SEEDS = range(6)


@pytest.fixture(scope="module")
def reference():
    from oracle.build import reference_available
    if not reference_available():
        pytest.skip("reference sources absent")
    from oracle.reference import Reference
    return Reference()


def _params(oracle, rng, n, b):
    r = float(rng.uniform(0.004, 0.02))
    return oracle.derive_params(r, float(rng.uniform(950, 1050)), n, b, float(rng.uniform(5e-4, 2e-3)),
                                float(rng.uniform(-12, 0)), float(rng.uniform(1e-7, 1e-4)), float(rng.uniform(0, 1.5)))


@pytest.mark.parametrize("seed", SEEDS)
def test_keys_permutation_ranges(oracle, reference, seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 5000))
    p = _params(oracle, rng, n, 0)
    cell = p.kernel_radius
    pos = (rng.standard_normal((n, 3)) * 8 * cell).astype(np.float32)
    pos[: n // 4] = (np.round(pos[: n // 4] / cell) * cell).astype(np.float32)  # exactly on cell borders
    k_o, s_o = oracle.initialize(p, pos)
    k_r, s_r = reference.initialize(p, pos)
    np.testing.assert_array_equal(k_o, k_r)
    np.testing.assert_array_equal(s_o, s_r)
    ks_r, ss_r = reference.stable_sort(k_r, s_r)
    ks_o, ss_o = oracle.counting_sort(k_o, s_o, p.bucket_count)
    np.testing.assert_array_equal(ks_o, ks_r)
    np.testing.assert_array_equal(ss_o, ss_r)
    vel = rng.standard_normal((n, 3)).astype(np.float32)
    po, vo, off_o = oracle.reorder(ks_o, ss_o, pos, vel, p.bucket_count)
    pr, vr, off_r = reference.reorder_fluid(p, ks_r, ss_r, pos, vel)
    np.testing.assert_array_equal(po, pr)
    np.testing.assert_array_equal(vo, vr)
    np.testing.assert_array_equal(off_o.reshape(-1), off_r.reshape(-1))


@pytest.mark.parametrize("seed", SEEDS)
def test_full_steps_random_scenes(oracle, reference, seed):
    from pcisph_gb300 import scenes
    rng = np.random.default_rng(100 + seed)
    side = int(rng.integers(5, 10))
    d = float(rng.uniform(0.01, 0.03))
    pos = scenes.lattice_block(side, side + 2, side, d, (0, 0, 0), seed=seed)
    b_pos = scenes.boundary_box((0, 0, 0), (side * d * 1.5, side * d * 3, side * d * 1.5), d, layers=1) \
        if seed % 2 else np.zeros((0, 3), np.float32)
    n, b = pos.shape[0], b_pos.shape[0]
    p = oracle.derive_params(0.5 * d, 1000.0, n, b, 1e-3 * d / 0.02, -9.81, float(rng.uniform(1e-7, 1e-5)),
                             float(rng.uniform(0.0, 1.0)))
    vel = (rng.standard_normal((n, 3)) * 0.05).astype(np.float32)
    so = oracle.new_state(p, pos, vel, b_pos)
    sr = oracle.new_state(p, pos, vel, b_pos)
    opts = make_options(threshold=0.01, min_iters=3, max_iters=7, walls=False, boundary_self_density=0)
    for k in range(3):
        st = oracle.step(p, opts, so, boundary_sort=(k == 0))
        it, me = reference.step(p, 0.01, 7, k == 0, 0, sr)
        assert st.iterations == it and np.float32(st.max_err) == np.float32(me), (k, st.iterations, it)
        for name in ("f_pos", "f_vel", "f_rho", "f_press", "f_src", "b_press"):
            np.testing.assert_array_equal(so[name], sr[name], err_msg=f"step {k} {name}")
