"""ctypes binding of libpcisph_gb300.so (the C ABI in include/pcisph_gpu.h).

The library is the only compute path: there is no CPU fallback. Loading fails
with an error naming the missing file when the library was not built.
"""
import ctypes as C
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libpcisph_gb300.so")
HEADER = os.path.join(ROOT, "include", "pcisph_gpu.h")

# status codes
OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_INCONSISTENT, ERR_NOT_READY, ERR_TIMEOUT = range(7)
STEP_NOT_CONVERGED, STEP_NONFINITE = 1, 2
LAYOUT_PACKED3, LAYOUT_FLOAT4, LAYOUT_SCALAR = 0, 1, 2
MEM_HOST, MEM_DEVICE = 0, 1
LIST_SKIN_ADAPTIVE = -1.0  # pcisph_batch_set_list_skin: each scene picks its skin every step
FIELDS = {
    "position": 0, "velocity": 1, "normal": 2, "predicted_position": 3, "density": 4, "other_force": 5,
    "pressure": 6, "pressure_force": 7, "density_variation": 8, "sorted_position": 9, "sorted_velocity": 10,
    "keys": 11, "src": 12, "cell_offsets": 13, "boundary_position": 14, "boundary_pressure": 15,
    "boundary_init_density": 16, "boundary_keys": 17, "boundary_src": 18, "boundary_cell_offsets": 19,
}
VECTOR_FIELDS = {"position", "velocity", "normal", "predicted_position", "other_force", "pressure_force",
                 "sorted_position", "sorted_velocity", "boundary_position"}
UINT_FIELDS = {"keys", "src", "cell_offsets", "boundary_keys", "boundary_src", "boundary_cell_offsets"}
STAGES = {"sort": 0, "density": 1, "normal": 2, "force": 3, "boundary_pressure": 4, "pressure": 5,
          "pressure_force": 6, "pack": 7, "boundary_pressure_reset": 8}


class SimParams(C.Structure):
    """pcisph_sim_params: mirror of Simulation_Params (PCISPH/data/kernels/Simulation_Params.h:18-44)."""
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
    _fields_ = [("min_iterations", C.c_int32), ("max_iterations", C.c_int32), ("walls", C.c_int32),
                ("box_lo", C.c_float * 3), ("box_hi", C.c_float * 3), ("restitution", C.c_float),
                ("boundary_self_density", C.c_int32), ("loop_mode", C.c_int32), ("kernel_variant", C.c_int32),
                ("list_skin", C.c_float), ("spatial_order", C.c_int32), ("sweep_block", C.c_int32),
                ("particle_skin", C.c_int32)]


class StepStats(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("max_density_error", C.c_float), ("status", C.c_uint32),
                ("status_all", C.c_uint32), ("steps", C.c_uint64), ("total_iterations", C.c_uint64),
                ("list_fallbacks", C.c_uint64), ("fast_particles", C.c_uint64), ("list_skin", C.c_float),
                ("max_density_error_max", C.c_float), ("unconverged_steps", C.c_uint64)]


class SceneDesc(C.Structure):
    """pcisph_scene_desc: one scene of a batch."""
    _fields_ = [("fluid_count", C.c_uint32), ("particle_radius", C.c_float), ("rest_density", C.c_float),
                ("delta_t", C.c_float), ("gravity", C.c_float), ("viscosity", C.c_float),
                ("surface_tension", C.c_float), ("density_variation_threshold", C.c_float),
                ("min_iterations", C.c_int32), ("max_iterations", C.c_int32), ("walls", C.c_int32),
                ("box_lo", C.c_float * 3), ("box_hi", C.c_float * 3), ("restitution", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("target", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_x_degrees", C.c_float)]


class TuneResult(C.Structure):
    _fields_ = [("list_skin", C.c_float), ("spatial_order", C.c_int32), ("digit_bits", C.c_int32),
                ("sweep_block", C.c_int32),
                ("ms_per_step", C.c_float), ("ms_per_step_before", C.c_float), ("candidates", C.c_int32)]


class BatchTuneResult(C.Structure):
    _fields_ = [("list_skin", C.c_float), ("loop_mode", C.c_int32), ("digit_bits", C.c_int32),
                ("ms_per_step", C.c_float), ("ms_per_step_before", C.c_float), ("candidates", C.c_int32)]


class KernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint64), ("total_ms", C.c_double)]


class PcisphError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"pcisph error {code}: {message}")
        self.code = code


_LIB = None


def header_functions():
    """Names of every function declared in include/pcisph_gpu.h."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"PCISPH_API\s+[\w\s\*]+?\b(pcisph_\w+)\s*\(", text)))


def load():
    """Load the CUDA library; raises if it is missing (no fallback exists)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with pcisph_gb300.build.build() "
                          "(the PCISPH step has no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    vp, u32, f32, i32, sz = C.c_void_p, C.c_uint32, C.c_float, C.c_int, C.c_size_t
    sig = {
        "pcisph_abi_version": ([], i32),
        "pcisph_last_error": ([], C.c_char_p),
        "pcisph_derive_params": ([f32, f32, u32, u32, f32, f32, f32, f32, C.POINTER(SimParams)], i32),
        "pcisph_sort_bit_count": ([u32], u32),
        "pcisph_default_options": ([C.POINTER(Options)], i32),
        "pcisph_create": ([i32, vp, C.POINTER(vp)], i32),
        "pcisph_destroy": ([vp], None),
        "pcisph_set_stream": ([vp, vp], i32),
        "pcisph_set_boundary_count": ([vp, u32], i32),
        "pcisph_set_fluid_count": ([vp, u32], i32),
        "pcisph_set_delta_t": ([vp, f32], i32),
        "pcisph_set_rest_density": ([vp, f32], i32),
        "pcisph_set_particle_radius": ([vp, f32], i32),
        "pcisph_set_gravity": ([vp, f32], i32),
        "pcisph_set_viscosity": ([vp, f32], i32),
        "pcisph_set_surface_tension": ([vp, f32], i32),
        "pcisph_set_density_variation_threshold": ([vp, f32], i32),
        "pcisph_set_options": ([vp, C.POINTER(Options)], i32),
        "pcisph_get_options": ([vp, C.POINTER(Options)], i32),
        "pcisph_get_params": ([vp, C.POINTER(SimParams)], i32),
        "pcisph_prepare": ([vp], i32),
        "pcisph_set_fluid_state": ([vp, vp, vp, u32, i32, i32], i32),
        "pcisph_set_boundary_state": ([vp, vp, u32, i32, i32], i32),
        "pcisph_check_buffers_consistent": ([vp], i32),
        "pcisph_update": ([vp], i32),
        "pcisph_step": ([vp, u32], i32),
        "pcisph_sync": ([vp], i32),
        "pcisph_sync_for": ([vp, C.c_int64], i32),
        "pcisph_last_stats": ([vp, C.POINTER(StepStats)], i32),
        "pcisph_reset_stats": ([vp], i32),
        "pcisph_get_field": ([vp, i32, vp, sz, i32, i32], i32),
        "pcisph_get_fluid_state": ([vp, vp, vp, u32, i32, i32], i32),
        "pcisph_set_field": ([vp, i32, vp, sz, i32, i32], i32),
        "pcisph_field_device_ptr": ([vp, i32, C.POINTER(vp), C.POINTER(sz), C.POINTER(i32)], i32),
        "pcisph_run_stage": ([vp, i32, i32], i32),
        "pcisph_render": ([vp, vp, C.c_uint32, C.c_float, C.c_float, C.POINTER(Camera), i32, i32, vp, sz, vp, vp],
                          i32),
        "pcisph_render_fluid": ([vp, C.POINTER(Camera), i32, i32, vp, sz], i32),
        "pcisph_autotune": ([vp, C.c_uint32, C.POINTER(TuneResult)], i32),
        "pcisph_snapshot_size": ([vp, C.POINTER(sz)], i32),
        "pcisph_snapshot": ([vp, vp, sz], i32),
        "pcisph_restore": ([vp, vp, sz], i32),
        "pcisph_kernel_launches": ([vp], C.c_uint64),
        "pcisph_profile_enable": ([vp, i32], i32),
        "pcisph_profile_read": ([vp, C.POINTER(KernelTime), i32, C.POINTER(i32)], i32),
        "pcisph_hash_keys": ([C.POINTER(SimParams), vp, i32, u32, vp, vp, vp], i32),
        "pcisph_radixsort_create": ([i32, C.POINTER(vp)], i32),
        "pcisph_radixsort_destroy": ([vp], None),
        "pcisph_radixsort_enqueue": ([vp, vp, vp, sz, C.c_uint, vp], i32),
        "pcisph_radixsort_set_digit_bits": ([vp, i32], i32),
        "pcisph_radixsort_enqueue_noalloc": ([vp, vp, sz, C.c_uint, vp], i32),
        "pcisph_batch_create": ([i32, vp, u32, u32, C.POINTER(vp)], i32),
        "pcisph_batch_destroy": ([vp], None),
        "pcisph_batch_memory_model": ([C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], i32),
        "pcisph_batch_add_scene": ([vp, C.POINTER(SceneDesc), vp, vp, i32, i32, C.POINTER(C.c_int32)], i32),
        "pcisph_batch_remove_scene": ([vp, C.c_int32], i32),
        "pcisph_batch_info": ([vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)], i32),
        "pcisph_batch_step": ([vp, u32], i32),
        "pcisph_batch_sync": ([vp], i32),
        "pcisph_batch_profile_enable": ([vp, i32], i32),
        "pcisph_batch_profile_read": ([vp, C.POINTER(KernelTime), i32, C.POINTER(i32)], i32),
        "pcisph_batch_sync_for": ([vp, C.c_int64], i32),
        "pcisph_batch_scene_stats": ([vp, C.c_int32, C.POINTER(StepStats)], i32),
        "pcisph_batch_get_field": ([vp, C.c_int32, i32, vp, sz, i32, i32], i32),
        "pcisph_batch_set_state": ([vp, C.c_int32, vp, vp, C.c_uint32, i32, i32], i32),
        "pcisph_batch_set_loop_mode": ([vp, i32], i32),
        "pcisph_batch_set_list_skin": ([vp, C.c_float], i32),
        "pcisph_batch_autotune": ([vp, C.c_uint32, C.POINTER(BatchTuneResult)], i32),
        "pcisph_batch_graph_stats": ([vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], i32),
        "pcisph_batch_kernel_launches": ([vp], C.c_uint64),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    if L.pcisph_abi_version() != 1:
        raise ImportError("libpcisph_gb300.so ABI version mismatch")
    _LIB = L
    return L


def check(rc):
    if rc != OK:
        msg = load().pcisph_last_error()
        raise PcisphError(rc, msg.decode() if msg else "")
    return rc
