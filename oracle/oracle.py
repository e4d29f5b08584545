"""ctypes wrapper of the oracle restatement (``pcisph_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``. Arrays are numpy, vectors packed ``(n, 3)``
(the reference layout). Every function mirrors one reference kernel or host
routine; the C++ source cites the reference line for each.
"""
import ctypes as C

import numpy as np

from .build import build_oracle

u32p = C.POINTER(C.c_uint32)
f32p = C.POINTER(C.c_float)
f64p = C.POINTER(C.c_double)


class SimParams(C.Structure):
    """Simulation_Params (PCISPH/data/kernels/Simulation_Params.h:18-44), 80 bytes."""
    _fields_ = [
        ("particle_radius", C.c_float), ("particle_mass", C.c_float), ("rest_density", C.c_float),
        ("boundary_count", C.c_uint32), ("fluid_count", C.c_uint32),
        ("kernel_radius", C.c_float), ("kernel_radius2", C.c_float),
        ("bucket_count", C.c_uint32), ("cell_size", C.c_float),
        ("poly6_normalization", C.c_float), ("poly6_d1_normalization", C.c_float),
        ("viscosity_d2_normalization", C.c_float), ("spiky_d1_normalization", C.c_float),
        ("surface_tension_coefficient", C.c_float), ("surface_tension_term", C.c_float),
        ("surface_tension_normalization", C.c_float),
        ("viscosity_constant", C.c_float), ("gravity", C.c_float), ("delta_t", C.c_float),
        ("density_variation_scaling_factor", C.c_float),
    ]


class Options(C.Structure):
    _fields_ = [("threshold", C.c_float), ("min_iters", C.c_int), ("max_iters", C.c_int), ("walls", C.c_int),
                ("box_lo", C.c_float * 3), ("box_hi", C.c_float * 3), ("restitution", C.c_float),
                ("boundary_self_density", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("max_err", C.c_float), ("converged", C.c_int)]


def make_options(threshold=0.01, min_iters=3, max_iters=7, walls=False, box_lo=(0, 0, 0), box_hi=(0, 0, 0),
                 restitution=0.5, boundary_self_density=0):
    o = Options()
    o.threshold, o.min_iters, o.max_iters, o.walls = threshold, min_iters, max_iters, int(bool(walls))
    o.box_lo[:] = [float(v) for v in box_lo]
    o.box_hi[:] = [float(v) for v in box_hi]
    o.restitution, o.boundary_self_density = restitution, int(boundary_self_density)
    return o


_STATE_F = ["f_pos", "f_vel", "f_normal", "f_pred", "f_rho", "f_other", "f_press", "f_fpress", "f_err",
            "b_pos", "b_press", "b_init"]
_STATE_U = ["f_keys", "f_src", "f_off", "b_keys", "b_src", "b_off"]


def _state_struct(ptype):
    class St(C.Structure):
        _fields_ = [(n, ptype) for n in _STATE_F] + [(n, u32p) for n in _STATE_U]
    return St


_StateF32 = _state_struct(f32p)
_StateF64 = _state_struct(f64p)


def _ptr(a, t):
    if a is None:
        return None
    assert a.flags.c_contiguous
    return a.ctypes.data_as(t)


def _f(a):
    return _ptr(a, f32p)


def _u(a):
    return _ptr(a, u32p)


class Oracle:
    def __init__(self):
        self.lib = C.CDLL(build_oracle())
        L = self.lib
        assert L.or_sizeof_params() == 80 and L.or_sizeof_params() == C.sizeof(SimParams)
        assert L.or_sizeof_options() == C.sizeof(Options)
        L.or_num_threads.restype = C.c_int
        L.or_derive_params.argtypes = [C.c_float, C.c_float, C.c_uint32, C.c_uint32, C.c_float, C.c_float,
                                       C.c_float, C.c_float, C.POINTER(SimParams)]
        L.or_sort_bit_count.argtypes = [C.c_uint32]
        L.or_sort_bit_count.restype = C.c_uint32
        L.or_hash_key.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32]
        L.or_hash_key.restype = C.c_uint32
        L.or_cell_pos.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_int)]
        P = C.POINTER(SimParams)
        L.or_initialize.argtypes = [P, C.c_uint32, f32p, u32p, u32p]
        L.or_counting_sort.argtypes = [u32p, u32p, C.c_uint32, C.c_uint32]
        L.or_reorder.argtypes = [C.c_uint32, C.c_uint32, u32p, u32p, f32p, f32p, f32p, f32p, u32p]
        L.or_update_density.argtypes = [P, u32p, f32p, u32p, f32p, f32p]
        L.or_update_normal.argtypes = [P, u32p, f32p, f32p, f32p]
        L.or_force_init.argtypes = [P, u32p, f32p, f32p, f32p, f32p, f32p, f32p, f32p]
        L.or_advance.argtypes = [P, C.POINTER(Options), f32p, f32p, f32p, f32p, f32p, f32p]
        L.or_boundary_self_density.argtypes = [P, u32p, f32p, f32p]
        L.or_update_pressure.argtypes = [P, C.c_int, u32p, f32p, f32p, u32p, f32p, f32p, f32p, f32p]
        L.or_pressure_force.argtypes = [P, u32p, f32p, f32p, u32p, f32p, f32p, f32p, f32p]
        L.or_step_f32.argtypes = [P, C.POINTER(Options), C.POINTER(_StateF32), C.c_int, C.POINTER(Stats)]
        L.or_step_f64.argtypes = [P, C.POINTER(Options), C.POINTER(_StateF64), C.c_int, C.POINTER(Stats)]
        L.or_force_init_f64.argtypes = [P, u32p, f64p, f64p, f64p, f64p, f64p, f64p, f64p]

    def num_threads(self):
        """OpenMP threads of the oracle's parallel loops."""
        return self.lib.or_num_threads()

    # -- params -----------------------------------------------------------
    def derive_params(self, particle_radius, rest_density, fluid_count, boundary_count, delta_t, gravity,
                      viscosity, surface_tension):
        p = SimParams()
        self.lib.or_derive_params(particle_radius, rest_density, fluid_count, boundary_count, delta_t, gravity,
                                  viscosity, surface_tension, C.byref(p))
        return p

    def sort_bit_count(self, n):
        return self.lib.or_sort_bit_count(n)

    # -- hashing / sort ---------------------------------------------------
    def hash_key(self, x, y, z, bk):
        return self.lib.or_hash_key(int(x), int(y), int(z), int(bk))

    def cell_pos(self, px, py, pz, cell):
        out = (C.c_int * 3)()
        self.lib.or_cell_pos(px, py, pz, cell, out)
        return tuple(out)

    def initialize(self, p, pos):
        pos = np.ascontiguousarray(pos, np.float32)
        n = pos.shape[0]
        keys = np.empty(n, np.uint32)
        src = np.empty(n, np.uint32)
        self.lib.or_initialize(C.byref(p), n, _f(pos), _u(keys), _u(src))
        return keys, src

    def counting_sort(self, keys, vals, bk):
        keys = np.ascontiguousarray(keys, np.uint32).copy()
        vals = np.ascontiguousarray(vals, np.uint32).copy()
        self.lib.or_counting_sort(_u(keys), _u(vals), keys.size, bk)
        return keys, vals

    def reorder(self, keys, src, pos, vel, bk):
        n = keys.size
        out_pos = np.empty((n, 3), np.float32)
        out_vel = np.empty((n, 3), np.float32) if vel is not None else None
        off = np.empty(2 * bk, np.uint32)
        self.lib.or_reorder(n, bk, _u(keys), _u(src), _f(np.ascontiguousarray(pos, np.float32)),
                            _f(None if vel is None else np.ascontiguousarray(vel, np.float32)), _f(out_pos),
                            _f(out_vel), _u(off))
        return out_pos, out_vel, off

    # -- kernels (FP32) ---------------------------------------------------
    def update_density(self, p, b_off, b_pos, f_off, f_pos):
        rho = np.empty(p.fluid_count, np.float32)
        self.lib.or_update_density(C.byref(p), _u(b_off), _f(b_pos), _u(f_off), _f(f_pos), _f(rho))
        return rho

    def update_normal(self, p, f_off, f_pos, rho):
        n = np.empty((p.fluid_count, 3), np.float32)
        self.lib.or_update_normal(C.byref(p), _u(f_off), _f(f_pos), _f(rho), _f(n))
        return n

    def force_init(self, p, f_off, pos, nrm, rho, vel):
        N = p.fluid_count
        fo, pr, fp = np.empty((N, 3), np.float32), np.empty(N, np.float32), np.empty((N, 3), np.float32)
        self.lib.or_force_init(C.byref(p), _u(f_off), _f(pos), _f(nrm), _f(rho), _f(vel), _f(fo), _f(pr), _f(fp))
        return fo, pr, fp

    def force_init_f64(self, p, f_off, pos, nrm, rho, vel):
        """force_init in FP64 on the same inputs (converted exactly from FP32)."""
        N = p.fluid_count
        d = lambda a: np.ascontiguousarray(a, np.float64)  # noqa: E731
        pos, nrm, rho, vel = d(pos), d(nrm), d(rho), d(vel)
        fo, pr, fp = np.empty((N, 3)), np.empty(N), np.empty((N, 3))
        self.lib.or_force_init_f64(C.byref(p), _u(f_off), _ptr(pos, f64p), _ptr(nrm, f64p), _ptr(rho, f64p),
                                   _ptr(vel, f64p), _ptr(fo, f64p), _ptr(pr, f64p), _ptr(fp, f64p))
        return fo, pr, fp

    def advance(self, p, pos, vel, f_other, f_press, integrate, options=None):
        N = p.fluid_count
        new_pos = np.empty((N, 3), np.float32)
        new_vel = np.empty((N, 3), np.float32) if integrate else None
        o = C.byref(options) if options is not None else None
        self.lib.or_advance(C.byref(p), o, _f(pos), _f(vel), _f(f_other), _f(f_press), _f(new_pos), _f(new_vel))
        return (new_pos, new_vel) if integrate else new_pos

    def boundary_self_density(self, p, b_off, b_pos):
        out = np.empty(p.boundary_count, np.float32)
        self.lib.or_boundary_self_density(C.byref(p), _u(b_off), _f(b_pos), _f(out))
        return out

    def update_pressure(self, p, boundary_update, b_off, b_pos, b_init, f_off, f_pos, f_pred, press_in,
                        want_err=True):
        press = np.array(press_in, np.float32, copy=True)
        err = np.empty(p.fluid_count, np.float32) if (want_err and not boundary_update) else None
        self.lib.or_update_pressure(C.byref(p), int(boundary_update), _u(b_off), _f(b_pos), _f(b_init), _u(f_off),
                                    _f(f_pos), _f(f_pred), _f(err), _f(press))
        return press, err

    def pressure_force(self, p, b_off, b_pos, b_press, f_off, f_pos, rho, press):
        fp = np.empty((p.fluid_count, 3), np.float32)
        self.lib.or_pressure_force(C.byref(p), _u(b_off), _f(b_pos), _f(b_press), _u(f_off), _f(f_pos), _f(rho),
                                   _f(press), _f(fp))
        return fp

    # -- full step --------------------------------------------------------
    def new_state(self, p, f_pos, f_vel, b_pos=None, dtype=np.float32):
        """Arrays for one scene; b_pos must already be sorted unless the step sorts it."""
        N, B, bk = p.fluid_count, p.boundary_count, p.bucket_count
        s = {
            "f_pos": np.array(f_pos, dtype).reshape(N, 3), "f_vel": np.array(f_vel, dtype).reshape(N, 3),
            "f_normal": np.zeros((N, 3), dtype), "f_pred": np.zeros((N, 3), dtype), "f_rho": np.zeros(N, dtype),
            "f_other": np.zeros((N, 3), dtype), "f_press": np.zeros(N, dtype), "f_fpress": np.zeros((N, 3), dtype),
            "f_err": np.zeros(N, dtype),
            "b_pos": np.array(b_pos if b_pos is not None else np.zeros((0, 3)), dtype).reshape(B, 3),
            "b_press": np.zeros(B, dtype), "b_init": np.zeros(B, dtype),
            "f_keys": np.zeros(N, np.uint32), "f_src": np.zeros(N, np.uint32), "f_off": np.zeros(2 * bk, np.uint32),
            "b_keys": np.zeros(B, np.uint32), "b_src": np.zeros(B, np.uint32), "b_off": np.zeros(2 * bk, np.uint32),
        }
        return s

    def step(self, p, options, state, boundary_sort=True):
        """One time step in place on ``state`` (see new_state). Precision follows the arrays' dtype."""
        f64 = state["f_pos"].dtype == np.float64
        St, fp = (_StateF64, f64p) if f64 else (_StateF32, f32p)
        st = St(**{n: _ptr(state[n], fp) for n in _STATE_F}, **{n: _ptr(state[n], u32p) for n in _STATE_U})
        stats = Stats()
        fn = self.lib.or_step_f64 if f64 else self.lib.or_step_f32
        fn(C.byref(p), C.byref(options), C.byref(st), int(bool(boundary_sort)), C.byref(stats))
        return stats


_ORACLE = None


def get():
    global _ORACLE
    if _ORACLE is None:
        _ORACLE = Oracle()
    return _ORACLE
