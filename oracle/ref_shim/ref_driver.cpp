/*
 * ref_driver.cpp -- host driver for the reference's own OpenCL kernels compiled
 * as C++ (see cl_shim.h). TEST INFRASTRUCTURE ONLY: the library this builds
 * (oracle/_ref/libpcisph_ref.so) generates golden vectors under tests/golden/
 * and pins the oracle restatement; the product never links it.
 *
 * This file is appended to the reference kernels in ONE translation unit by
 * oracle/build_ref.sh, so the kernels below are called directly. Each
 * ref_<kernel>() runs one NDRange: an OpenMP loop in which every iteration is
 * one work-item (cl_shim_global_id), which is how a CPU OpenCL runtime maps an
 * NDRange onto host threads. ref_step() restates the host sequence of
 * sim::Fluid::update() (PCISPH/src/sim/Fluid.cpp:108-327) with
 * std::stable_sort standing in for clogs::Radixsort::enqueue (its contract:
 * stable key/value sort, libs/clogs/include/clogs/radixsort.h:176-185).
 */
#include <algorithm>
#include <numeric>
#include <vector>
#include <cstring>

thread_local size_t cl_shim_global_id = 0;

#define REF_NDRANGE(count, call)                      \
    do {                                              \
        long long _n = (long long)(count);            \
        _Pragma("omp parallel for schedule(static)")  \
        for (long long _g = 0; _g < _n; ++_g) {       \
            cl_shim_global_id = (size_t)_g;           \
            call;                                     \
        }                                             \
    } while (0)

extern "C" {

int ref_sizeof_params(void) { return (int)sizeof(Simulation_Params); }

/* The setters (Fluid.cpp:333-375) followed by update_deduced_attributes (:377-443). */
void ref_derive_params(float particle_radius, float rest_density, uint fluid_count, uint boundary_count,
                       float delta_t, float gravity, float viscosity, float surface_tension, Simulation_Params* out) {
    sim::Fluid f;
    std::memset(&f.params, 0, sizeof(f.params));
    f.params.particle_radius = particle_radius;
    f.params.rest_density = rest_density;
    f.params.fluid_count = fluid_count;
    f.params.boundary_count = boundary_count;
    f.params.delta_t = delta_t;
    f.params.gravity = gravity;
    f.params.viscosity_constant = viscosity;
    f.params.surface_tension_coefficient = surface_tension;
    f.update_deduced_attributes();
    *out = f.params;
}

/* sort_utils.cl:7-10 */
void ref_reset_cell_offsets(const Simulation_Params* p, uint* cell_offsets) {
    REF_NDRANGE(p->bucket_count, reset_cell_offsets(p, cell_offsets));
}

/* sort_utils.cl:12-23 */
void ref_initialize(const Simulation_Params* p, uint count, uint* keys, float* positions, uint* src) {
    REF_NDRANGE(count, initialize(p, count, keys, positions, src));
}

/* The clogs sort is a stable key/value sort (radixsort.h:183-185). */
void ref_stable_sort(uint* keys, uint* values, uint count) {
    std::vector<uint> order(count);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint a, uint b) { return keys[a] < keys[b]; });
    std::vector<uint> k(count), v(count);
    for (uint i = 0; i < count; ++i) { k[i] = keys[order[i]]; v[i] = values[order[i]]; }
    std::memcpy(keys, k.data(), count * sizeof(uint));
    std::memcpy(values, v.data(), count * sizeof(uint));
}

/* sort_utils.cl:25-49 */
void ref_reorder_boundary(uint count, uint* cell_offsets, uint* src, uint* keys, float* in_pos, float* out_pos) {
    REF_NDRANGE(count, reorder_and_insert_boundary_offsets(count, cell_offsets, src, keys, in_pos, out_pos));
}

/* sort_utils.cl:51-78 */
void ref_reorder_fluid(uint count, uint* cell_offsets, uint* src, uint* keys, float* in_pos, float* in_vel,
                       float* out_pos, float* out_vel) {
    REF_NDRANGE(count, reorder_and_insert_fluid_offsets(count, cell_offsets, src, keys, in_pos, in_vel, out_pos, out_vel));
}

/* pcisph.cl:65-92 */
void ref_update_density(const Simulation_Params* p, uint* b_off, float* b_pos, uint* f_off, float* f_pos, float* rho) {
    REF_NDRANGE(p->fluid_count, update_density(p, b_off, b_pos, f_off, f_pos, rho));
}

/* pcisph.cl:94-112 */
void ref_update_normal(const Simulation_Params* p, uint* f_off, float* f_pos, float* rho, float* normals) {
    REF_NDRANGE(p->fluid_count, update_normal(p, f_off, f_pos, rho, normals));
}

/* pcisph.cl:114-119 */
void ref_boundary_pressure_initialization(const Simulation_Params* p, float* b_press) {
    REF_NDRANGE(p->boundary_count, boundary_pressure_initialization(p, b_press));
}

/* pcisph.cl:121-173 */
void ref_force_initialization(const Simulation_Params* p, uint* f_off, float* pos, float* normals, float* rho,
                              float* vel, float* f_other, float* press, float* f_press) {
    REF_NDRANGE(p->fluid_count, force_initialization(p, f_off, pos, normals, rho, vel, f_other, press, f_press));
}

/* pcisph.cl:175-193; new_vel may be NULL (predict) */
void ref_update_position_and_velocity(const Simulation_Params* p, float* pos, float* vel, float* f_other,
                                      float* f_press, float* new_pos, float* new_vel) {
    REF_NDRANGE(p->fluid_count, update_position_and_velocity(p, pos, vel, f_other, f_press, new_pos, new_vel));
}

/* pcisph.cl:195-210 (never enqueued by the reference host, Fluid.cpp:167-171) */
void ref_initialize_boundary_boundary_pred_densities(const Simulation_Params* p, uint* b_off, float* b_pos, float* out) {
    REF_NDRANGE(p->boundary_count, initialize_boundary_boundary_pred_densities(p, b_off, b_pos, out));
}

/* pcisph.cl:212-263; err may be NULL */
void ref_update_pressure(const Simulation_Params* p, int boundary_update, uint* b_off, float* b_pos, float* b_init,
                         uint* f_off, float* f_pos, float* f_pred, float* err, float* out_press) {
    uint count = boundary_update ? p->boundary_count : p->fluid_count;
    REF_NDRANGE(count, update_pressure(p, boundary_update, b_off, b_pos, b_init, f_off, f_pos, f_pred, err, out_press));
}

/* pcisph.cl:265-300 */
void ref_update_pressure_force(const Simulation_Params* p, uint* b_off, float* b_pos, float* b_press, uint* f_off,
                               float* f_pos, float* rho, float* press, float* f_press) {
    REF_NDRANGE(p->fluid_count, update_pressure_force(p, b_off, b_pos, b_press, f_off, f_pos, rho, press, f_press));
}

/*
 * One time step in the order of Fluid::update (Fluid.cpp:108-327).
 *   boundary_sort          sort the boundary set this step (the reference does so
 *                          once after a parameter change, Fluid.cpp:135-174)
 *   boundary_self_density  0: boundary_init_pred_densities stays zero (the kernel is
 *                          never enqueued, Fluid.cpp:167-171); 1: run it
 * The step's internal buffers (keys, src, cell tables, err) are caller-owned so that
 * a test can read them. b_off must hold 2*bucket_count entries even when
 * boundary_count == 0 (it is then all zero). Returns the iteration count.
 */
int ref_step(const Simulation_Params* p, float threshold, int max_iters, int boundary_sort, int boundary_self_density,
             float* b_pos, float* b_press, float* b_init, uint* b_off, uint* b_keys, uint* b_src, float* b_tmp,
             float* f_pos, float* f_vel, float* f_normals, float* f_pred, float* f_rho, float* f_other,
             float* f_press, float* f_fpress, uint* f_off, uint* f_keys, uint* f_src, float* f_pos_tmp,
             float* f_vel_tmp, float* f_err, float* out_max_err) {
    const uint N = p->fluid_count, B = p->boundary_count;
    if (N == 0) return 0;
    if (boundary_sort && B > 0) {
        ref_reset_cell_offsets(p, b_off);
        ref_initialize(p, B, b_keys, b_pos, b_src);
        ref_stable_sort(b_keys, b_src, B);
        std::memcpy(b_tmp, b_pos, 3 * (size_t)B * sizeof(float));
        ref_reorder_boundary(B, b_off, b_src, b_keys, b_tmp, b_pos);
        if (boundary_self_density) ref_initialize_boundary_boundary_pred_densities(p, b_off, b_pos, b_init);
        else std::memset(b_init, 0, (size_t)B * sizeof(float));
    }
    ref_reset_cell_offsets(p, f_off);
    ref_initialize(p, N, f_keys, f_pos, f_src);
    ref_stable_sort(f_keys, f_src, N);
    std::memcpy(f_pos_tmp, f_pos, 3 * (size_t)N * sizeof(float));
    std::memcpy(f_vel_tmp, f_vel, 3 * (size_t)N * sizeof(float));
    ref_reorder_fluid(N, f_off, f_src, f_keys, f_pos_tmp, f_vel_tmp, f_pos, f_vel);

    ref_update_density(p, b_off, b_pos, f_off, f_pos, f_rho);
    ref_update_normal(p, f_off, f_pos, f_rho, f_normals);
    if (B > 0) ref_boundary_pressure_initialization(p, b_press);
    ref_force_initialization(p, f_off, f_pos, f_normals, f_rho, f_vel, f_other, f_press, f_fpress);

    const int min_iterations = 2;
    int iters = 0;
    float max_err = 0.f;
    for (int i = 0; i < max_iters; i++) {
        ref_update_position_and_velocity(p, f_pos, f_vel, f_other, f_fpress, f_pred, nullptr);
        if (B > 0) ref_update_pressure(p, 1, b_off, b_pos, b_init, f_off, f_pos, f_pred, nullptr, b_press);
        ref_update_pressure(p, 0, b_off, b_pos, b_init, f_off, f_pos, f_pred, f_err, f_press);
        ref_update_pressure_force(p, b_off, b_pos, b_press, f_off, f_pos, f_rho, f_press, f_fpress);
        iters = i + 1;
        max_err = *std::max_element(f_err, f_err + N);
        if (i >= min_iterations && max_err / p->rest_density < threshold) break;
    }
    ref_update_position_and_velocity(p, f_pos, f_vel, f_other, f_fpress, f_pos, f_vel);
    if (out_max_err) *out_max_err = max_err;
    return iters;
}

}  // extern "C"
