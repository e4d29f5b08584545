"""Helpers shared by the GPU parity tests."""
import ctypes as C

import numpy as np

from pcisph_gb300 import Fluid
from pcisph_gb300._lib import SimParams

# FP32 parity bound for one kernel on identical inputs, normwise: |gpu - ref| <= RTOL * scale, where scale is
# the magnitude of the terms summed (by default the largest magnitude in the field). Summation terms of mixed
# sign (normals, forces) are compared on that scale, never component by component on a near-zero value.
RTOL = 1e-5


def params_from(b):
    p = SimParams()
    C.memmove(C.addressof(p), bytes(np.asarray(b, np.uint8)), C.sizeof(SimParams))
    return p


def rel_err(got, want, scale=None):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    if scale is None:
        scale = np.abs(want).max() if want.size else 1.0
    scale = max(float(scale), 1e-30)
    return float(np.abs(got - want).max() / scale) if want.size else 0.0


def assert_close(name, got, want, scale=None, rtol=RTOL):
    e = rel_err(got, want, scale)
    assert e <= rtol, f"{name}: normwise relative error {e:.3e} > {rtol:.0e}"
    return e


def fluid_like(p, min_iters=3, max_iters=7, walls=False, box_lo=(0, 0, 0), box_hi=(0, 0, 0), restitution=0.5,
               boundary_self_density=0, loop_mode=0, threshold=0.01, kernel_variant=2, spatial_order=1):
    """A context configured through the reference setters for params p (as scene::load does)."""
    f = Fluid(0)
    f.set_delta_t(p.delta_t)
    f.set_rest_density(p.rest_density)
    f.set_viscosity(p.viscosity_constant)
    f.set_surface_tension(p.surface_tension_coefficient)
    f.set_gravity(p.gravity)
    f.set_density_variation_threshold(threshold)
    f.set_particle_radius(p.particle_radius)
    f.set_fluid_count(p.fluid_count)
    f.set_boundary_count(p.boundary_count)
    f.set_options(min_iterations=min_iters, max_iterations=max_iters, walls=int(walls), box_lo=box_lo,
                  box_hi=box_hi, restitution=restitution, boundary_self_density=boundary_self_density,
                  loop_mode=loop_mode, kernel_variant=kernel_variant, spatial_order=spatial_order)
    f.prepare()
    return f


def kinetic_energy(m, vel):
    v = np.asarray(vel, np.float64)
    return 0.5 * m * float((v * v).sum())
