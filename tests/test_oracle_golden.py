"""Pin the oracle restatement to golden vectors from the reference's own kernels.

The golden files were produced by tests/golden/make_golden.py, which runs the
reference's OpenCL kernels and parameter derivation compiled on the host. The
oracle follows the same arithmetic expression by expression, so every integer
result and every FP32 field must match bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.oracle import SimParams, make_options


def params_from(b):
    p = SimParams()
    C.memmove(C.addressof(p), bytes(np.asarray(b, np.uint8)), C.sizeof(SimParams))
    return p


def test_params_match_reference(oracle, golden):
    g = golden("params")
    for row, want in zip(g["inputs"], g["params"]):
        r, rho0, n, b, dt, grav, mu, gam = row
        p = oracle.derive_params(np.float32(r), np.float32(rho0), int(n), int(b), np.float32(dt), np.float32(grav),
                                 np.float32(mu), np.float32(gam))
        got = np.frombuffer(bytes(p), np.float32)
        ref = np.frombuffer(bytes(want), np.float32)
        # the derivation calls powf/pow; allow 1 ulp between libm implementations
        assert np.all(np.abs(got.view(np.int32).astype(np.int64) - ref.view(np.int32).astype(np.int64)) <= 1), row
        gi, ri = np.frombuffer(bytes(p), np.uint32), np.frombuffer(bytes(want), np.uint32)
        for idx in (3, 4, 7):  # boundary_count, fluid_count, bucket_count are integers
            assert gi[idx] == ri[idx]


def test_sort_bit_count(oracle, golden):
    for n in golden("params")["sort_bits_n"]:
        n = int(n)
        # Fluid.cpp:125-133: smallest b with 2^b - 1 >= n - 1 (n = 0 wraps to 2^32 - 1)
        want = next(i + 1 for i in range(32) if (2 ** (i + 1) - 1) >= ((n - 1) % 2 ** 32))
        assert oracle.sort_bit_count(n) == want


def test_hash_keys_bit_exact(oracle, golden):
    g = golden("hash")
    for name in g:
        if not name.startswith("keys_"):
            continue
        p = SimParams()
        p.cell_size = g["cell"]
        p.bucket_count = int(name[5:])
        keys, src = oracle.initialize(p, g["pos"])
        np.testing.assert_array_equal(keys, g[name])
        np.testing.assert_array_equal(src, np.arange(len(keys)))


def test_stable_sort_bit_exact(oracle, golden):
    g = golden("sort")
    i = 0
    while f"keys_{i}" in g:
        keys = g[f"keys_{i}"]
        bk = int(keys.max()) + 1
        sk, sv = oracle.counting_sort(keys, np.arange(keys.size, dtype=np.uint32), bk)
        np.testing.assert_array_equal(sk, g[f"sorted_keys_{i}"])
        np.testing.assert_array_equal(sv, g[f"sorted_vals_{i}"])
        i += 1


@pytest.mark.parametrize("case", ["step_boundary", "step_fluid", "step_dambreak"])
def test_kernel_chain_bit_exact(oracle, golden, case):
    g = golden(case)
    p = params_from(g["params"])
    N, B, bk = p.fluid_count, p.boundary_count, p.bucket_count
    eq = np.testing.assert_array_equal
    if B:
        keys, src = oracle.initialize(p, g["b_pos0"])
        keys, src = oracle.counting_sort(keys, src, bk)
        eq(keys, g["b_keys"]); eq(src, g["b_src"])
        b_pos, _, b_off = oracle.reorder(keys, src, g["b_pos0"], None, bk)
        eq(b_pos, g["b_pos"]); eq(b_off, g["b_off"])
        eq(oracle.boundary_self_density(p, b_off, b_pos), g["b_init"])
    else:
        b_pos, b_off = np.zeros((0, 3), np.float32), np.zeros(2 * bk, np.uint32)
    keys, src = oracle.initialize(p, g["f_pos0"])
    eq(keys, g["f_keys_unsorted"])
    keys, src = oracle.counting_sort(keys, src, bk)
    eq(keys, g["f_keys"]); eq(src, g["f_src"])
    f_pos, f_vel, f_off = oracle.reorder(keys, src, g["f_pos0"], g["f_vel0"], bk)
    eq(f_pos, g["f_pos"]); eq(f_vel, g["f_vel"]); eq(f_off, g["f_off"])
    rho = oracle.update_density(p, b_off, b_pos, f_off, f_pos)
    eq(rho, g["rho"])
    nrm = oracle.update_normal(p, f_off, f_pos, rho)
    eq(nrm, g["normal"])
    fo, pr, fp = oracle.force_init(p, f_off, f_pos, nrm, rho, f_vel)
    eq(fo, g["f_other"]); eq(pr, 0); eq(fp, 0)
    b_press = np.zeros(B, np.float32)
    zeros_b = np.zeros(B, np.float32)
    for it in range(2):
        pred = oracle.advance(p, f_pos, f_vel, fo, fp, integrate=False)
        eq(pred, g[f"pred{it}"])
        if B:
            b_press, _ = oracle.update_pressure(p, 1, b_off, b_pos, zeros_b, f_off, f_pos, pred, b_press)
            eq(b_press, g[f"b_press{it}"])
            bpc, _ = oracle.update_pressure(p, 1, b_off, b_pos, g["b_init"], f_off, f_pos, pred, zeros_b)
            eq(bpc, g[f"b_press_computed{it}_from0"])
        eq(pr, g[f"press_in{it}"])
        pr, err = oracle.update_pressure(p, 0, b_off, b_pos, zeros_b, f_off, f_pos, pred, pr)
        eq(pr, g[f"press{it}"]); eq(err, g[f"err{it}"])
        fp = oracle.pressure_force(p, b_off, b_pos, b_press, f_off, f_pos, rho, pr)
        eq(fp, g[f"fpress{it}"])
    x1, v1 = oracle.advance(p, f_pos, f_vel, fo, fp, integrate=True)
    eq(x1, g["x_new"]); eq(v1, g["v_new"])


@pytest.mark.parametrize("case", ["step_boundary", "step_fluid", "step_dambreak"])
def test_full_steps_bit_exact(oracle, golden, case):
    """Fluid::update sequence: reference settings (min 3, max 7 iterations, no walls, zero boundary self density)."""
    g = golden(case)
    p = params_from(g["params"])
    s = oracle.new_state(p, g["f_pos0"], g["f_vel0"], g["b_pos0"])
    opts = make_options(threshold=0.01, min_iters=3, max_iters=7, walls=False, boundary_self_density=0)
    k = 0
    while f"step{k}_iters" in g:
        st = oracle.step(p, opts, s, boundary_sort=(k == 0))
        assert st.iterations == int(g[f"step{k}_iters"])
        assert np.float32(st.max_err) == g[f"step{k}_max_err"]
        for n in ("f_pos", "f_vel", "f_normal", "f_pred", "f_rho", "f_other", "f_press", "f_fpress", "f_err",
                  "f_src", "b_press"):
            np.testing.assert_array_equal(s[n], g[f"step{k}_{n}"], err_msg=f"{case} step {k} {n}")
        k += 1
    np.testing.assert_array_equal(s["b_pos"], g["b_pos_sorted"])


def test_fp64_step_close_to_fp32(oracle, golden):
    """The FP64 rerun of a step stays close to FP32 (the FP32 error is what the GPU tests are scaled by)."""
    g = golden("step_fluid")
    p = params_from(g["params"])
    opts = make_options(threshold=0.01, min_iters=3, max_iters=3)
    s32 = oracle.new_state(p, g["f_pos0"], g["f_vel0"])
    s64 = oracle.new_state(p, g["f_pos0"], g["f_vel0"], dtype=np.float64)
    oracle.step(p, opts, s32)
    oracle.step(p, opts, s64)
    np.testing.assert_array_equal(s32["f_src"], s64["f_src"])
    np.testing.assert_allclose(s32["f_rho"], s64["f_rho"], rtol=1e-5)
    np.testing.assert_allclose(s32["f_pos"], s64["f_pos"], rtol=0, atol=1e-6)
