// pcisph_fluid.hpp -- header-only C++ mirror of the reference's sim::Fluid over the C ABI.
//
// Same method names and meaning as PCISPH/src/sim/Fluid.h:13-29: the nine setters mark the parameters
// changed, update() re-derives them when needed (zeroing the velocities, Fluid.cpp:377-466), checks the
// state against the counts (Fluid.cpp:90-106) and advances one time step (Fluid.cpp:108-327). Errors
// surface as std::runtime_error, as in the reference (Fluid.cpp:95, :132). The reference's public
// cl::Buffer members become set_*_state() imports and field() exports; device_ptr() replaces the
// CL-GL shared buffers.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "pcisph_gpu.h"

namespace pcisph {

inline void check(int rc) {
    if (rc != PCISPH_OK) throw std::runtime_error(std::string("pcisph: ") + pcisph_last_error());
}

class Fluid {
   public:
    explicit Fluid(int device = 0, void* cuda_stream = nullptr) { check(pcisph_create(device, cuda_stream, &ctx_)); }
    ~Fluid() { pcisph_destroy(ctx_); }
    Fluid(const Fluid&) = delete;
    Fluid& operator=(const Fluid&) = delete;
    Fluid(Fluid&& o) noexcept : ctx_(o.ctx_) { o.ctx_ = nullptr; }

    // Fluid.h:16-18
    void checkBuffersConsistent() const { check(pcisph_check_buffers_consistent(ctx_)); }
    void update() { check(pcisph_update(ctx_)); }
    pcisph_sim_params get_params() const {
        pcisph_sim_params p;
        check(pcisph_get_params(ctx_, &p));
        return p;
    }

    // Fluid.h:21-29
    void set_boundary_count(unsigned int n) { check(pcisph_set_boundary_count(ctx_, n)); }
    void set_fluid_count(unsigned int n) { check(pcisph_set_fluid_count(ctx_, n)); }
    void set_delta_t(float v) { check(pcisph_set_delta_t(ctx_, v)); }
    void set_rest_density(float v) { check(pcisph_set_rest_density(ctx_, v)); }
    void set_particle_radius(float v) { check(pcisph_set_particle_radius(ctx_, v)); }
    void set_gravity(float v) { check(pcisph_set_gravity(ctx_, v)); }
    void set_viscosity(float v) { check(pcisph_set_viscosity(ctx_, v)); }
    void set_surface_tension(float v) { check(pcisph_set_surface_tension(ctx_, v)); }
    void set_density_variation_threshold(float v) { check(pcisph_set_density_variation_threshold(ctx_, v)); }

    // Options the reference fixes in code (iterations 3..7, no walls); defaults reproduce it.
    pcisph_options options() const {
        pcisph_options o;
        check(pcisph_get_options(ctx_, &o));
        return o;
    }
    void set_options(const pcisph_options& o) { check(pcisph_set_options(ctx_, &o)); }
    void prepare() { check(pcisph_prepare(ctx_)); }

    // State, packed xyz per particle (the reference's vload3 layout) from host memory.
    void set_fluid_state(const std::vector<float>& pos, const std::vector<float>& vel) {
        check(pcisph_set_fluid_state(ctx_, pos.data(), vel.empty() ? nullptr : vel.data(),
                                     static_cast<uint32_t>(pos.size() / 3), PCISPH_LAYOUT_PACKED3, PCISPH_MEM_HOST));
    }
    void set_boundary_state(const std::vector<float>& pos) {
        check(pcisph_set_boundary_state(ctx_, pos.data(), static_cast<uint32_t>(pos.size() / 3),
                                        PCISPH_LAYOUT_PACKED3, PCISPH_MEM_HOST));
    }
    // Positions and velocities back into caller buffers of count x 3 floats, one synchronisation (pinned
    // buffers are written directly by the device).
    void get_fluid_state(float* pos, float* vel, uint32_t count) {
        check(pcisph_get_fluid_state(ctx_, pos, vel, count, PCISPH_LAYOUT_PACKED3, PCISPH_MEM_HOST));
    }
    // A field copied to the host: vectors packed xyz, scalars one value per particle.
    std::vector<float> field(pcisph_field f) {
        void* p = nullptr;
        size_t n = 0;
        int layout = 0;
        check(pcisph_field_device_ptr(ctx_, f, &p, &n, &layout));
        const int out_layout = layout == PCISPH_LAYOUT_FLOAT4 ? PCISPH_LAYOUT_PACKED3 : PCISPH_LAYOUT_SCALAR;
        std::vector<float> out(n * (out_layout == PCISPH_LAYOUT_PACKED3 ? 3 : 1));
        check(pcisph_get_field(ctx_, f, out.data(), out.size() * sizeof(float), out_layout, PCISPH_MEM_HOST));
        return out;
    }
    // Zero-copy device view (float4 per particle for vectors), e.g. for CUDA-GL interop by a renderer.
    void* device_ptr(pcisph_field f, size_t* count = nullptr) {
        void* p = nullptr;
        check(pcisph_field_device_ptr(ctx_, f, &p, count, nullptr));
        return p;
    }
    pcisph_step_stats stats() {
        pcisph_step_stats s;
        check(pcisph_last_stats(ctx_, &s));
        return s;
    }
    void sync() { check(pcisph_sync(ctx_)); }
    pcisph_ctx* handle() { return ctx_; }

   private:
    pcisph_ctx* ctx_ = nullptr;
};

}  // namespace pcisph
