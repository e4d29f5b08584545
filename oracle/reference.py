"""ctypes wrapper of the reference's own kernels compiled on the host (``_ref/``).

TEST INFRASTRUCTURE ONLY. Available only where the reference sources exist
(``build.build_reference``); used to generate ``tests/golden/`` and, when
present, to check the oracle directly. Each ``ref_*`` symbol runs one reference
kernel as an NDRange (see ``ref_shim/ref_driver.cpp``).
"""
import ctypes as C
import os

import numpy as np

from .build import build_reference
from .oracle import SimParams, _f, _u, f32p, u32p


class Reference:
    def __init__(self, path=None):
        path = path or build_reference()
        if path is None:
            raise FileNotFoundError("reference kernels are not built and their sources are absent")
        self.lib = C.CDLL(path)
        L = self.lib
        assert L.ref_sizeof_params() == 80
        P = C.POINTER(SimParams)
        L.ref_reset_cell_offsets.argtypes = [P, u32p]
        L.ref_initialize.argtypes = [P, C.c_uint, u32p, f32p, u32p]
        L.ref_stable_sort.argtypes = [u32p, u32p, C.c_uint]
        L.ref_reorder_boundary.argtypes = [C.c_uint, u32p, u32p, u32p, f32p, f32p]
        L.ref_reorder_fluid.argtypes = [C.c_uint, u32p, u32p, u32p, f32p, f32p, f32p, f32p]
        L.ref_update_density.argtypes = [P, u32p, f32p, u32p, f32p, f32p]
        L.ref_update_normal.argtypes = [P, u32p, f32p, f32p, f32p]
        L.ref_boundary_pressure_initialization.argtypes = [P, f32p]
        L.ref_force_initialization.argtypes = [P, u32p, f32p, f32p, f32p, f32p, f32p, f32p, f32p]
        L.ref_update_position_and_velocity.argtypes = [P, f32p, f32p, f32p, f32p, f32p, f32p]
        L.ref_initialize_boundary_boundary_pred_densities.argtypes = [P, u32p, f32p, f32p]
        L.ref_update_pressure.argtypes = [P, C.c_int, u32p, f32p, f32p, u32p, f32p, f32p, f32p, f32p]
        L.ref_update_pressure_force.argtypes = [P, u32p, f32p, f32p, u32p, f32p, f32p, f32p, f32p]
        L.ref_step.argtypes = [P, C.c_float, C.c_int, C.c_int, C.c_int,
                               f32p, f32p, f32p, u32p, u32p, u32p, f32p,
                               f32p, f32p, f32p, f32p, f32p, f32p, f32p, f32p, u32p, u32p, u32p, f32p, f32p, f32p,
                               f32p]
        L.ref_step.restype = C.c_int
        L.ref_derive_params.argtypes = [C.c_float, C.c_float, C.c_uint, C.c_uint, C.c_float, C.c_float,
                                        C.c_float, C.c_float, P]

    def derive_params(self, particle_radius, rest_density, fluid_count, boundary_count, delta_t, gravity, viscosity,
                      surface_tension):
        """Setters + Fluid::update_deduced_attributes compiled from the reference (Fluid.cpp:377-443)."""
        p = SimParams()
        self.lib.ref_derive_params(particle_radius, rest_density, fluid_count, boundary_count, delta_t, gravity,
                                   viscosity, surface_tension, C.byref(p))
        return p

    def initialize(self, p, pos):
        pos = np.ascontiguousarray(pos, np.float32)
        n = pos.shape[0]
        keys, src = np.empty(n, np.uint32), np.empty(n, np.uint32)
        self.lib.ref_initialize(C.byref(p), n, _u(keys), _f(pos), _u(src))
        return keys, src

    def stable_sort(self, keys, vals):
        keys, vals = np.array(keys, np.uint32), np.array(vals, np.uint32)
        self.lib.ref_stable_sort(_u(keys), _u(vals), keys.size)
        return keys, vals

    def reorder_fluid(self, p, keys, src, pos, vel):
        n = keys.size
        off = np.empty(2 * p.bucket_count, np.uint32)
        self.lib.ref_reset_cell_offsets(C.byref(p), _u(off))
        op, ov = np.empty((n, 3), np.float32), np.empty((n, 3), np.float32)
        self.lib.ref_reorder_fluid(n, _u(off), _u(src), _u(keys), _f(np.ascontiguousarray(pos, np.float32)),
                                   _f(np.ascontiguousarray(vel, np.float32)), _f(op), _f(ov))
        return op, ov, off

    def reorder_boundary(self, p, keys, src, pos):
        n = keys.size
        off = np.empty(2 * p.bucket_count, np.uint32)
        self.lib.ref_reset_cell_offsets(C.byref(p), _u(off))
        op = np.empty((n, 3), np.float32)
        self.lib.ref_reorder_boundary(n, _u(off), _u(src), _u(keys), _f(np.ascontiguousarray(pos, np.float32)),
                                      _f(op))
        return op, off

    def update_density(self, p, b_off, b_pos, f_off, f_pos):
        rho = np.empty(p.fluid_count, np.float32)
        self.lib.ref_update_density(C.byref(p), _u(b_off), _f(b_pos), _u(f_off), _f(f_pos), _f(rho))
        return rho

    def update_normal(self, p, f_off, f_pos, rho):
        n = np.empty((p.fluid_count, 3), np.float32)
        self.lib.ref_update_normal(C.byref(p), _u(f_off), _f(f_pos), _f(rho), _f(n))
        return n

    def force_init(self, p, f_off, pos, nrm, rho, vel):
        N = p.fluid_count
        fo, pr, fp = np.empty((N, 3), np.float32), np.empty(N, np.float32), np.empty((N, 3), np.float32)
        self.lib.ref_force_initialization(C.byref(p), _u(f_off), _f(pos), _f(nrm), _f(rho), _f(vel), _f(fo), _f(pr),
                                          _f(fp))
        return fo, pr, fp

    def advance(self, p, pos, vel, f_other, f_press, integrate):
        N = p.fluid_count
        if integrate:
            new_pos, new_vel = np.array(pos, np.float32), np.array(vel, np.float32)
            self.lib.ref_update_position_and_velocity(C.byref(p), _f(new_pos), _f(new_vel), _f(f_other),
                                                      _f(f_press), _f(new_pos), _f(new_vel))
            return new_pos, new_vel
        new_pos = np.empty((N, 3), np.float32)
        self.lib.ref_update_position_and_velocity(C.byref(p), _f(pos), _f(vel), _f(f_other), _f(f_press),
                                                  _f(new_pos), None)
        return new_pos

    def boundary_self_density(self, p, b_off, b_pos):
        out = np.empty(p.boundary_count, np.float32)
        self.lib.ref_initialize_boundary_boundary_pred_densities(C.byref(p), _u(b_off), _f(b_pos), _f(out))
        return out

    def update_pressure(self, p, boundary_update, b_off, b_pos, b_init, f_off, f_pos, f_pred, press_in):
        press = np.array(press_in, np.float32, copy=True)
        err = None if boundary_update else np.empty(p.fluid_count, np.float32)
        self.lib.ref_update_pressure(C.byref(p), int(boundary_update), _u(b_off), _f(b_pos), _f(b_init), _u(f_off),
                                     _f(f_pos), _f(f_pred), _f(err), _f(press))
        return press, err

    def pressure_force(self, p, b_off, b_pos, b_press, f_off, f_pos, rho, press):
        fp = np.empty((p.fluid_count, 3), np.float32)
        self.lib.ref_update_pressure_force(C.byref(p), _u(b_off), _f(b_pos), _f(b_press), _u(f_off), _f(f_pos),
                                           _f(rho), _f(press), _f(fp))
        return fp

    def step(self, p, threshold, max_iters, boundary_sort, boundary_self_density, s):
        """Fluid::update on state dict ``s`` (see oracle.Oracle.new_state plus b_tmp/f_pos_tmp/f_vel_tmp)."""
        N, B = p.fluid_count, p.boundary_count
        tmp = {"b_tmp": np.zeros((max(B, 1), 3), np.float32), "f_pos_tmp": np.zeros((N, 3), np.float32),
               "f_vel_tmp": np.zeros((N, 3), np.float32)}
        me = C.c_float(0)
        it = self.lib.ref_step(C.byref(p), threshold, max_iters, int(boundary_sort), int(boundary_self_density),
                               _f(s["b_pos"]), _f(s["b_press"]), _f(s["b_init"]), _u(s["b_off"]), _u(s["b_keys"]),
                               _u(s["b_src"]), _f(tmp["b_tmp"]),
                               _f(s["f_pos"]), _f(s["f_vel"]), _f(s["f_normal"]), _f(s["f_pred"]), _f(s["f_rho"]),
                               _f(s["f_other"]), _f(s["f_press"]), _f(s["f_fpress"]), _u(s["f_off"]),
                               _u(s["f_keys"]), _u(s["f_src"]), _f(tmp["f_pos_tmp"]), _f(tmp["f_vel_tmp"]),
                               _f(s["f_err"]), C.byref(me))
        return it, me.value


def load_xraw_reference(path, particles_per_dimension, scaling):
    """The reference's own scene loader (scenes.cpp:76-149, compiled by build_ref.sh into
    libpcisph_ref_scene.so): (fluid, boundary, visible cubes) positions, each (n, 3) float32."""
    lib_path = os.path.join(os.path.dirname(build_reference() or ""), "libpcisph_ref_scene.so")
    L = C.CDLL(lib_path)
    fp, ul = C.POINTER(C.c_float), C.c_ulong
    L.ref_load_xraw.argtypes = [C.c_char_p, C.c_uint, C.c_float, C.POINTER(fp), C.POINTER(ul), C.POINTER(fp),
                                C.POINTER(ul), C.POINTER(fp), C.POINTER(ul)]
    L.ref_free.argtypes = [C.c_void_p]
    ptrs, counts = [fp() for _ in range(3)], [ul() for _ in range(3)]
    rc = L.ref_load_xraw(str(path).encode(), int(particles_per_dimension), C.c_float(scaling),
                         C.byref(ptrs[0]), C.byref(counts[0]), C.byref(ptrs[1]), C.byref(counts[1]),
                         C.byref(ptrs[2]), C.byref(counts[2]))
    if rc:
        raise FileNotFoundError(path)
    out = []
    for ptr, n in zip(ptrs, counts):
        out.append(np.ctypeslib.as_array(ptr, (n.value * 3,)).reshape(-1, 3).copy() if n.value
                   else np.zeros((0, 3), np.float32))
        L.ref_free(ptr)
    return tuple(out)
