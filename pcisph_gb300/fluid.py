"""Python mirror of the reference's simulation interface, over the C ABI.

``Fluid`` has the methods of sim::Fluid (PCISPH/src/sim/Fluid.h:13-29):
``update()``, ``get_params()``, ``check_buffers_consistent()`` and the nine
setters, with the same semantics (a setter marks the parameters changed; the
next update re-derives them and zeroes the velocities, Fluid.cpp:377-466).
The reference's public cl::Buffers become properties and ``get_field`` /
``set_field`` calls. Host arrays are numpy; device arrays are anything with a
``data_ptr()`` (torch tensors) and are passed as device pointers.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import FIELDS, STAGES, UINT_FIELDS, VECTOR_FIELDS, check, load


def _is_device(a):
    return hasattr(a, "data_ptr") and getattr(a, "is_cuda", False)


def _ptr(a):
    if a is None:
        return None
    if _is_device(a):
        return C.c_void_p(a.data_ptr())
    assert isinstance(a, np.ndarray) and a.flags.c_contiguous
    return C.c_void_p(a.ctypes.data)


def _layout_of(a):
    shape = tuple(a.shape)
    if len(shape) == 2 and shape[1] == 4:
        return _lib.LAYOUT_FLOAT4
    if len(shape) == 2 and shape[1] == 3:
        return _lib.LAYOUT_PACKED3
    raise ValueError(f"vector arrays must be (n, 3) or (n, 4), got {shape}")


def derive_params(particle_radius, rest_density, fluid_count, boundary_count, delta_t, gravity, viscosity,
                  surface_tension):
    """Setters + Fluid::update_deduced_attributes as a pure host computation."""
    p = _lib.SimParams()
    check(load().pcisph_derive_params(particle_radius, rest_density, fluid_count, boundary_count, delta_t, gravity,
                                      viscosity, surface_tension, C.byref(p)))
    return p


def default_options():
    o = _lib.Options()
    check(load().pcisph_default_options(C.byref(o)))
    return o


class Fluid:
    """One simulation context on one GPU (sim::Fluid, Fluid.h:13-102)."""

    def __init__(self, device=0, stream=None):
        L = load()
        h = C.c_void_p()
        check(L.pcisph_create(int(device), C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h
        self._L = L

    def close(self):
        if getattr(self, "_h", None):
            self._L.pcisph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- reference setters (Fluid.h:21-29) ---------------------------------
    def set_boundary_count(self, n): check(self._L.pcisph_set_boundary_count(self._h, int(n)))
    def set_fluid_count(self, n): check(self._L.pcisph_set_fluid_count(self._h, int(n)))
    def set_delta_t(self, v): check(self._L.pcisph_set_delta_t(self._h, float(v)))
    def set_rest_density(self, v): check(self._L.pcisph_set_rest_density(self._h, float(v)))
    def set_particle_radius(self, v): check(self._L.pcisph_set_particle_radius(self._h, float(v)))
    def set_gravity(self, v): check(self._L.pcisph_set_gravity(self._h, float(v)))
    def set_viscosity(self, v): check(self._L.pcisph_set_viscosity(self._h, float(v)))
    def set_surface_tension(self, v): check(self._L.pcisph_set_surface_tension(self._h, float(v)))
    def set_density_variation_threshold(self, v):
        check(self._L.pcisph_set_density_variation_threshold(self._h, float(v)))

    def get_params(self):
        p = _lib.SimParams()
        check(self._L.pcisph_get_params(self._h, C.byref(p)))
        return p

    def set_options(self, **kw):
        o = _lib.Options()
        check(self._L.pcisph_get_options(self._h, C.byref(o)))
        for k, v in kw.items():
            if k in ("box_lo", "box_hi"):
                getattr(o, k)[:] = [float(x) for x in v]
            else:
                setattr(o, k, v)
        check(self._L.pcisph_set_options(self._h, C.byref(o)))

    def get_options(self):
        o = _lib.Options()
        check(self._L.pcisph_get_options(self._h, C.byref(o)))
        return o

    def set_stream(self, stream):
        check(self._L.pcisph_set_stream(self._h, C.c_void_p(stream) if stream else None))

    def prepare(self):
        check(self._L.pcisph_prepare(self._h))

    # -- state ---------------------------------------------------------------
    def set_fluid_state(self, pos, vel=None):
        n = int(pos.shape[0])
        mem = _lib.MEM_DEVICE if _is_device(pos) else _lib.MEM_HOST
        if mem == _lib.MEM_HOST:
            pos = np.ascontiguousarray(pos, np.float32)
            vel = None if vel is None else np.ascontiguousarray(vel, np.float32)
        check(self._L.pcisph_set_fluid_state(self._h, _ptr(pos), _ptr(vel), n, _layout_of(pos), mem))

    def set_boundary_state(self, pos):
        n = int(pos.shape[0])
        mem = _lib.MEM_DEVICE if _is_device(pos) else _lib.MEM_HOST
        if mem == _lib.MEM_HOST:
            pos = np.ascontiguousarray(pos, np.float32).reshape(n, 3 if pos.size == 3 * n else 4)
        check(self._L.pcisph_set_boundary_state(self._h, _ptr(pos), n, _layout_of(pos), mem))

    def check_buffers_consistent(self):
        check(self._L.pcisph_check_buffers_consistent(self._h))

    # -- stepping ---------------------------------------------------------------
    def update(self):
        """Fluid::update: one time step (stream-ordered)."""
        check(self._L.pcisph_update(self._h))

    def step(self, n):
        check(self._L.pcisph_step(self._h, int(n)))

    def sync(self, timeout_ms=None):
        """Wait for the queued steps; with timeout_ms, raise PcisphError (code ERR_TIMEOUT) if they are
        still running after that many milliseconds (the work stays queued)."""
        if timeout_ms is None:
            check(self._L.pcisph_sync(self._h))
        else:
            check(self._L.pcisph_sync_for(self._h, int(timeout_ms)))

    def stats(self):
        s = _lib.StepStats()
        check(self._L.pcisph_last_stats(self._h, C.byref(s)))
        return s

    def reset_stats(self):
        check(self._L.pcisph_reset_stats(self._h))

    def autotune(self, steps=3):
        """Pick the fastest list skin / working order / sort digit width, then the corrective-loop sweeps'
        block size, on the current state (results are unchanged by any choice); returns the choice and the
        step times."""
        r = _lib.TuneResult()
        check(self._L.pcisph_autotune(self._h, int(steps), C.byref(r)))
        return {"list_skin": r.list_skin, "spatial_order": r.spatial_order, "digit_bits": r.digit_bits,
                "sweep_block": r.sweep_block,
                "ms_per_step": r.ms_per_step, "ms_per_step_before": r.ms_per_step_before,
                "candidates": r.candidates}

    # -- checkpoints ----------------------------------------------------------
    def snapshot(self):
        """The context's parameters, options and state as bytes (pcisph_snapshot)."""
        n = C.c_size_t()
        check(self._L.pcisph_snapshot_size(self._h, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        check(self._L.pcisph_snapshot(self._h, buf, n.value))
        return buf.raw

    def restore(self, data):
        """Continue from a snapshot (pcisph_restore)."""
        buf = C.create_string_buffer(bytes(data), len(data))
        check(self._L.pcisph_restore(self._h, buf, len(data)))

    def save(self, path):
        """Write a checkpoint file (the snapshot bytes)."""
        with open(path, "wb") as f:
            f.write(self.snapshot())

    def load(self, path):
        with open(path, "rb") as f:
            self.restore(f.read())

    def run_stage(self, stage, arg=0):
        check(self._L.pcisph_run_stage(self._h, STAGES[stage], int(arg)))

    def kernel_launches(self):
        return int(self._L.pcisph_kernel_launches(self._h))

    def profile(self, enable=True):
        check(self._L.pcisph_profile_enable(self._h, int(bool(enable))))

    def profile_read(self):
        n = C.c_int()
        check(self._L.pcisph_profile_read(self._h, None, 0, C.byref(n)))
        arr = (_lib.KernelTime * max(1, n.value))()
        check(self._L.pcisph_profile_read(self._h, arr, n.value, C.byref(n)))
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(n.value)}

    # -- fields ---------------------------------------------------------------
    def _count(self, name):
        v, n, lay = C.c_void_p(), C.c_size_t(), C.c_int()
        check(self._L.pcisph_field_device_ptr(self._h, FIELDS[name], C.byref(v), C.byref(n), C.byref(lay)))
        return int(n.value)

    def device_ptr(self, name):
        """Zero-copy device view: (pointer, element count, native layout)."""
        v, n, lay = C.c_void_p(), C.c_size_t(), C.c_int()
        check(self._L.pcisph_field_device_ptr(self._h, FIELDS[name], C.byref(v), C.byref(n), C.byref(lay)))
        return v.value, int(n.value), int(lay.value)

    def get_field(self, name, layout="packed3", out=None):
        """Copy a field to a new numpy array ((n,3)/(n,4) for vectors, (n,) for scalars) or into ``out``."""
        n = self._count(name)
        if name in VECTOR_FIELDS:
            lay = _lib.LAYOUT_PACKED3 if layout == "packed3" else _lib.LAYOUT_FLOAT4
            shape, dt = (n, 3 if lay == _lib.LAYOUT_PACKED3 else 4), np.float32
        else:
            lay, shape, dt = _lib.LAYOUT_SCALAR, (n,), (np.uint32 if name in UINT_FIELDS else np.float32)
        if out is not None and _is_device(out):
            check(self._L.pcisph_get_field(self._h, FIELDS[name], _ptr(out), out.numel() * out.element_size(), lay,
                                           _lib.MEM_DEVICE))
            return out
        arr = out if out is not None else np.empty(shape, dt)
        check(self._L.pcisph_get_field(self._h, FIELDS[name], _ptr(arr), arr.nbytes, lay, _lib.MEM_HOST))
        return arr

    def get_fluid_state(self, pos=None, vel=None, layout="packed3"):
        """Positions and velocities in one call (one synchronisation), into ``pos`` / ``vel`` (numpy or
        device tensors of n x 3 or n x 4 floats) or new numpy arrays. Returns (pos, vel)."""
        n = self._count("position")
        lay = _lib.LAYOUT_PACKED3 if layout == "packed3" else _lib.LAYOUT_FLOAT4
        if pos is None:
            pos = np.empty((n, 3 if lay == _lib.LAYOUT_PACKED3 else 4), np.float32)
        if vel is None:
            vel = np.empty_like(pos)
        dev = _is_device(pos)
        if dev != _is_device(vel):
            raise ValueError("pos and vel must both be host arrays or both device tensors")
        for a in (pos, vel):
            if (a.numel() * a.element_size() if dev else a.nbytes) < n * (12 if lay == _lib.LAYOUT_PACKED3 else 16):
                raise ValueError("output too small")
        check(self._L.pcisph_get_fluid_state(self._h, _ptr(pos), _ptr(vel), n, lay,
                                             _lib.MEM_DEVICE if dev else _lib.MEM_HOST))
        return pos, vel

    def set_field(self, name, arr):
        if _is_device(arr):
            mem, nbytes = _lib.MEM_DEVICE, arr.numel() * arr.element_size()
        else:
            arr = np.ascontiguousarray(arr, np.uint32 if name in UINT_FIELDS else np.float32)
            mem, nbytes = _lib.MEM_HOST, arr.nbytes
        lay = _layout_of(arr) if name in VECTOR_FIELDS else _lib.LAYOUT_SCALAR
        check(self._L.pcisph_set_field(self._h, FIELDS[name], _ptr(arr), nbytes, lay, mem))

    # reference-style buffer properties (Fluid.h:40-50)
    @property
    def fluid_positions(self): return self.get_field("position")
    @property
    def fluid_velocities(self): return self.get_field("velocity")
    @property
    def fluid_normals(self): return self.get_field("normal")
    @property
    def fluid_predicted_positions(self): return self.get_field("predicted_position")
    @property
    def fluid_densities(self): return self.get_field("density")
    @property
    def fluid_other_forces(self): return self.get_field("other_force")
    @property
    def fluid_pressures(self): return self.get_field("pressure")
    @property
    def fluid_pressure_forces(self): return self.get_field("pressure_force")
    @property
    def boundary_positions(self): return self.get_field("boundary_position")
    @property
    def boundary_pressures(self): return self.get_field("boundary_pressure")


def setup_scene(fluid, scene, walls=None, loop_mode=0, max_iters=None, min_iters=None, boundary_self_density=0,
                kernel_variant=2, spatial_order=2):
    """Configure ``fluid`` for a scenes.Scene the way scene::load does (scenes.cpp:217-245)."""
    fluid.set_delta_t(scene.delta_t)
    fluid.set_rest_density(scene.rest_density)
    fluid.set_viscosity(scene.viscosity_constant())
    fluid.set_surface_tension(scene.surface_tension)
    fluid.set_gravity(scene.gravity)
    fluid.set_density_variation_threshold(scene.threshold)
    fluid.set_particle_radius(scene.particle_radius)
    fluid.set_fluid_count(scene.fluid_count)
    fluid.set_boundary_count(scene.boundary_count)
    fluid.set_options(min_iterations=scene.min_iters if min_iters is None else min_iters,
                      max_iterations=scene.max_iters if max_iters is None else max_iters,
                      walls=int(scene.walls if walls is None else walls), box_lo=scene.box_lo, box_hi=scene.box_hi,
                      restitution=scene.restitution, boundary_self_density=boundary_self_density,
                      loop_mode=loop_mode, kernel_variant=kernel_variant, spatial_order=spatial_order)
    fluid.prepare()
    fluid.set_fluid_state(scene.fluid_pos, scene.fluid_vel)
    if scene.boundary_count:
        fluid.set_boundary_state(scene.boundary_pos)


class RadixSort:
    """clogs::Radixsort replacement (radixsort.h:55-211) on device pointers."""

    def __init__(self, device=0, digit_bits=0):
        L = load()
        h = C.c_void_p()
        check(L.pcisph_radixsort_create(int(device), C.byref(h)))
        self._h, self._L = h, L
        if digit_bits:
            check(L.pcisph_radixsort_set_digit_bits(h, int(digit_bits)))

    def enqueue(self, keys, values, elements=None, max_bits=0, stream=None):
        n = keys.numel() if elements is None else int(elements)
        check(self._L.pcisph_radixsort_enqueue(self._h, _ptr(keys), _ptr(values), n, int(max_bits),
                                               C.c_void_p(stream) if stream else None))

    def close(self):
        if getattr(self, "_h", None):
            self._L.pcisph_radixsort_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def hash_keys(params, pos, keys, ids=None, stream=None):
    """sort_utils.cl:12-23 on device arrays: keys (and ids) of positions pos ((n,3) or (n,4))."""
    n = int(pos.shape[0])
    check(load().pcisph_hash_keys(C.byref(params), _ptr(pos), _layout_of(pos), n, _ptr(keys), _ptr(ids),
                                  C.c_void_p(stream) if stream else None))
