"""Many independent scenes advanced together (the pcisph_batch_* C ABI).

One launch per kernel per time step serves every scene; each scene keeps its own parameters and its own
convergence (it stops iterating when its own max density error is below its threshold). A scene's result
is the one it would have alone (tests/test_gpu_batch.py).
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import FIELDS, SceneDesc, StepStats, UINT_FIELDS, VECTOR_FIELDS, check, load


def scene_desc(scene, min_iters=None, max_iters=None):
    """pcisph_scene_desc for a scenes.Scene."""
    d = SceneDesc()
    d.fluid_count = scene.fluid_count
    d.particle_radius = scene.particle_radius
    d.rest_density = scene.rest_density
    d.delta_t = scene.delta_t
    d.gravity = scene.gravity
    d.viscosity = scene.viscosity_constant()
    d.surface_tension = scene.surface_tension
    d.density_variation_threshold = scene.threshold
    d.min_iterations = scene.min_iters if min_iters is None else min_iters
    d.max_iterations = scene.max_iters if max_iters is None else max_iters
    d.walls = int(scene.walls)
    d.box_lo[:] = [float(v) for v in scene.box_lo]
    d.box_hi[:] = [float(v) for v in scene.box_hi]
    d.restitution = scene.restitution
    return d


def memory_model():
    """(bytes per particle, bytes per scene) of a batch pool."""
    a, b = C.c_uint64(), C.c_uint64()
    check(load().pcisph_batch_memory_model(C.byref(a), C.byref(b)))
    return a.value, b.value


class Batch:
    def __init__(self, device=0, max_particles=1 << 20, max_scenes=256, stream=None, loop_mode=0):
        L = load()
        h = C.c_void_p()
        check(L.pcisph_batch_create(int(device), C.c_void_p(stream) if stream else None, int(max_particles),
                                    int(max_scenes), C.byref(h)))
        self._h, self._L = h, L
        if loop_mode:
            self.set_loop_mode(loop_mode)

    def close(self):
        if getattr(self, "_h", None):
            self._L.pcisph_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, scene, min_iters=None, max_iters=None, pos=None, vel=None):
        d = scene_desc(scene, min_iters, max_iters)
        pos = np.ascontiguousarray(scene.fluid_pos if pos is None else pos, np.float32)
        vel = scene.fluid_vel if vel is None else vel
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32)
        sid = C.c_int32()
        layout = _lib.LAYOUT_FLOAT4 if pos.shape[1] == 4 else _lib.LAYOUT_PACKED3
        check(self._L.pcisph_batch_add_scene(self._h, C.byref(d), C.c_void_p(pos.ctypes.data),
                                             None if vel is None else C.c_void_p(vel.ctypes.data), layout,
                                             _lib.MEM_HOST, C.byref(sid)))
        return sid.value

    def set_state(self, sid, pos, vel=None):
        """Replace a scene's state from host arrays ((n, 3) or (n, 4) float32; vel None: zero)."""
        pos = np.ascontiguousarray(pos, np.float32)
        vel = None if vel is None else np.ascontiguousarray(vel, np.float32)
        layout = _lib.LAYOUT_FLOAT4 if pos.shape[1] == 4 else _lib.LAYOUT_PACKED3
        if vel is not None and vel.shape != pos.shape:
            raise ValueError("positions and velocities differ in shape")
        check(self._L.pcisph_batch_set_state(self._h, int(sid), C.c_void_p(pos.ctypes.data),
                                             None if vel is None else C.c_void_p(vel.ctypes.data),
                                             pos.shape[0], layout, _lib.MEM_HOST))

    def autotune(self, steps=2):
        """Pick the fastest list skin / loop mode / sort digit width on the current scenes (results are
        unchanged by any choice); returns the choice and the step times."""
        r = _lib.BatchTuneResult()
        check(self._L.pcisph_batch_autotune(self._h, int(steps), C.byref(r)))
        skin = "adaptive" if r.list_skin == _lib.LIST_SKIN_ADAPTIVE else r.list_skin
        return {"list_skin": skin, "loop_mode": r.loop_mode, "digit_bits": r.digit_bits,
                "ms_per_step": r.ms_per_step, "ms_per_step_before": r.ms_per_step_before,
                "candidates": r.candidates}

    def set_loop_mode(self, mode):
        """0: the corrective loop as a graph WHILE node; 2: one persistent cooperative kernel."""
        check(self._L.pcisph_batch_set_loop_mode(self._h, int(mode)))

    def set_list_skin(self, skin):
        """Neighbour-list skin of every scene in units of h, or "adaptive" (the default: each scene picks
        0.25, 0.35 or 0.5 before each step from its previous step's displacements); results do not depend
        on it."""
        v = _lib.LIST_SKIN_ADAPTIVE if skin == "adaptive" else float(skin)
        check(self._L.pcisph_batch_set_list_skin(self._h, v))

    def remove_scene(self, sid):
        check(self._L.pcisph_batch_remove_scene(self._h, int(sid)))

    def info(self):
        a, b, c = C.c_uint32(), C.c_uint32(), C.c_uint32()
        check(self._L.pcisph_batch_info(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def step(self, n=1):
        check(self._L.pcisph_batch_step(self._h, int(n)))

    def profile(self, enable=True):
        """While enabled, steps run host-driven with every launch timed (same kernels, same results)."""
        check(self._L.pcisph_batch_profile_enable(self._h, int(bool(enable))))

    def profile_read(self):
        """{kernel name: (launches, total ms)} of the profiled steps."""
        n = C.c_int()
        check(self._L.pcisph_batch_profile_read(self._h, None, 0, C.byref(n)))
        arr = (_lib.KernelTime * max(1, n.value))()
        check(self._L.pcisph_batch_profile_read(self._h, arr, n.value, C.byref(n)))
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(n.value)}

    def sync(self, timeout_ms=None):
        """Wait for the queued steps; with timeout_ms, raise PcisphError (ERR_TIMEOUT) if they are still
        running after that many milliseconds (the work stays queued)."""
        if timeout_ms is None:
            check(self._L.pcisph_batch_sync(self._h))
        else:
            check(self._L.pcisph_batch_sync_for(self._h, int(timeout_ms)))

    def stats(self, sid):
        s = StepStats()
        check(self._L.pcisph_batch_scene_stats(self._h, int(sid), C.byref(s)))
        return s

    def graph_stats(self):
        """(step graphs instantiated, updated in place) since creation."""
        a, b = C.c_uint64(), C.c_uint64()
        check(self._L.pcisph_batch_graph_stats(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def kernel_launches(self):
        return int(self._L.pcisph_batch_kernel_launches(self._h))

    def get_field(self, sid, name, count, layout="packed3"):
        if name in VECTOR_FIELDS:
            lay = _lib.LAYOUT_PACKED3 if layout == "packed3" else _lib.LAYOUT_FLOAT4
            out = np.empty((count, 3 if lay == _lib.LAYOUT_PACKED3 else 4), np.float32)
        else:
            lay, out = _lib.LAYOUT_SCALAR, np.empty(count, np.uint32 if name in UINT_FIELDS else np.float32)
        check(self._L.pcisph_batch_get_field(self._h, int(sid), FIELDS[name], C.c_void_p(out.ctypes.data),
                                             out.nbytes, lay, _lib.MEM_HOST))
        return out
