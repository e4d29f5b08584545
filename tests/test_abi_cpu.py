"""The C ABI library builds, loads and exports every declared symbol; host-only calls work without a GPU."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from pcisph_gb300 import _lib, build, derive_params, scenes


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_exports_every_header_function(lib):
    declared = _lib.header_functions()
    assert len(declared) >= 40
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    # nothing but the ABI is exported
    extra = [s for s in exported if not s.startswith("pcisph_")]
    assert not extra, extra


def test_struct_sizes_match_header(lib):
    assert C.sizeof(_lib.SimParams) == 80  # Simulation_Params.h:18-44, packed
    o = _lib.Options()
    assert lib.pcisph_default_options(C.byref(o)) == 0
    assert (o.min_iterations, o.max_iterations, o.walls, o.boundary_self_density, o.loop_mode) == (3, 7, 0, 0, 0)


def test_derive_params_matches_oracle_bit_exact(lib, oracle):
    for args in [(0.01, 1000.0, 32768, 0, 1e-3, -9.81, 1.6e-6, 0.5),
                 (0.0025, 1000.0, 1 << 20, 0, 2.5e-4, -9.81, 2.5e-8, 0.5),
                 (0.00125, 1000.0, 1 << 23, 0, 1.25e-4, -9.81, 3.125e-9, 0.5),
                 (0.5 * 0.7 / 18, 999.972, 279936, 154980, 0.002, -9.81, 8e-5, 1.0),
                 (0.01, 1000.0, 1, 0, 1e-3, -9.81, 0.0, 0.0)]:
        assert bytes(derive_params(*args)) == bytes(oracle.derive_params(*args)), args


def test_derive_params_matches_reference_golden(lib, golden):
    g = golden("params")
    for row, want in zip(g["inputs"], g["params"]):
        r, rho0, n, b, dt, grav, mu, gam = row
        p = derive_params(np.float32(r), np.float32(rho0), int(n), int(b), np.float32(dt), np.float32(grav),
                          np.float32(mu), np.float32(gam))
        got = np.frombuffer(bytes(p), np.int32).astype(np.int64)
        ref = np.frombuffer(bytes(want), np.int32).astype(np.int64)
        assert np.all(np.abs(got - ref) <= 1), row  # <= 1 ulp across libm implementations


def test_sort_bit_count(lib):
    for n in [1, 2, 3, 4, 5, 63, 64, 65, 1000, 1 << 20, (1 << 20) + 1, 1 << 23]:
        want = next(i + 1 for i in range(32) if (2 ** (i + 1) - 1) >= n - 1)
        assert lib.pcisph_sort_bit_count(n) == want


def test_error_paths_without_gpu(lib):
    assert lib.pcisph_create(0, None, None) == _lib.ERR_INVALID_ARG
    assert b"NULL" in lib.pcisph_last_error()
    assert lib.pcisph_derive_params(0.01, 1000, 10, 0, 1e-3, 0, 0, 0, None) == _lib.ERR_INVALID_ARG
    assert lib.pcisph_update(None) == _lib.ERR_INVALID_ARG


def _magic(d):
    """Host restatement of common.cuh magic_for (Granlund-Montgomery, N = 31)."""
    ell = 0
    while (1 << ell) < d:
        ell += 1
    return ((1 << (31 + ell)) + d - 1) // d, ell - 1


@pytest.mark.parametrize("d", [64, 128, 192, 16384, 524288, 4194304, 64 * 999983, 2 ** 31 - 64, 1000000000])
def test_magic_modulo_exact(d):
    m, sh = _magic(d)
    assert m < 2 ** 32
    rng = np.random.default_rng(d)
    v = np.concatenate([rng.integers(0, 2 ** 31, 200000, dtype=np.int64),
                        np.arange(0, 4096), 2 ** 31 - 1 - np.arange(0, 4096),
                        (np.arange(1, 2000) * d) % (2 ** 31), (np.arange(1, 2000) * d - 1) % (2 ** 31)]).astype(np.uint64)
    q = ((v * np.uint64(m)) >> np.uint64(32)) >> np.uint64(sh)
    np.testing.assert_array_equal(q, v // np.uint64(d))


def test_scene_configs_are_deterministic():
    a, b = scenes.dam_break_32k(), scenes.dam_break_32k()
    assert a.fluid_count == 32768
    np.testing.assert_array_equal(a.fluid_pos, b.fluid_pos)
    assert a.fluid_pos.min() > 0 and a.fluid_pos.max() < 0.64
    jitter = a.fluid_pos - (np.floor(a.fluid_pos / 0.02) + 0.5) * 0.02
    assert np.abs(jitter).max() <= 0.05 * 0.02 * 1.0001
    c1 = scenes.dam_break(8, seed=0, extent=0.64)
    assert c1.fluid_count == 512 and abs(c1.spacing - 0.08) < 1e-12
    assert abs(scenes.dam_break_32k().viscosity_constant() - 0.2 * 0.02 ** 3) < 1e-15


def test_ctypes_structs_match_the_c_layout(tmp_path):
    """Every ctypes mirror in _lib has the size and field offsets the C compiler gives the header's struct
    (a field added on one side only would shift every later field)."""
    pairs = [(_lib.SimParams, "pcisph_sim_params"), (_lib.Options, "pcisph_options"),
             (_lib.StepStats, "pcisph_step_stats"), (_lib.SceneDesc, "pcisph_scene_desc"),
             (_lib.Camera, "pcisph_camera"), (_lib.TuneResult, "pcisph_tune_result"),
             (_lib.BatchTuneResult, "pcisph_batch_tune_result"), (_lib.KernelTime, "pcisph_kernel_time")]
    lines = ['#include <stddef.h>', '#include <stdio.h>', f'#include "{_lib.HEADER}"', "int main(void) {"]
    for cls, cname in pairs:
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for name, *_ in cls._fields_:
            lines.append(f'printf("{cname}.{name} %zu\\n", offsetof({cname}, {name}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for cls, cname in pairs:
        assert int(got[cname]) == C.sizeof(cls), cname
        for name, *_ in cls._fields_:
            assert int(got[f"{cname}.{name}"]) == getattr(cls, name).offset, (cname, name)
