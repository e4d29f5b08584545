// host_util.h -- host-side helpers shared by the step context (context.cu) and the batch (batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "../../include/pcisph_gpu.h"
#include "common.cuh"

namespace pcisph {

int report_error(int code, const std::string& msg);  // context.cu: sets pcisph_last_error()

namespace host {

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// The float whose bit pattern is b (a device-side float kept as bits for atomic max).
inline float float_from_bits(uint32_t b) {
    float f;
    std::memcpy(&f, &b, sizeof f);
    return f;
}

inline constexpr float kPi = 3.14159265358979323846f;  // utils/constants.h:4
inline constexpr uint32_t kListCap = 96;           // neighbour-list entries per particle (multiple of 4)
inline constexpr uint32_t kNearCap = 64;           // within-h list entries per particle
inline constexpr uint32_t kBoundaryListCap = 48;   // boundary particles within r_list per fluid particle
inline constexpr uint32_t kBoundaryFluidCap = 64;  // fluid particles within r_list per boundary particle
// partner marks: fast predictions a round may list (more: the round walks by bucket flags)
inline constexpr uint32_t kMarkCap = 65536;
// skin-list entries per particle of a batch (skins up to 0.5 h: ~48 (1 + skin)^3 entries at rest density)
inline constexpr uint32_t kListCapWide = 168;
// adaptive skin: a level qualifies if at most 1 in this many of the last step's predictions outran it
// (256 batched scenes, 9.8M particles, 500 steps: 27.1, 27.0, 27.1, 27.3 s at 500, 3000, 20000, 10^6)
inline constexpr uint32_t kSkinOutrunRatio = 500;
// per-particle skins: a particle's next half skin is kSkinFactor times its largest predicted displacement of
// the step, at least kSkinMinHalf h (measured at 1M: 0.00-0.05% of the predictions then outrun their skin)
inline constexpr float kSkinFactor = 2.0f;
inline constexpr float kSkinMinHalf = 0.02f;

// Wait up to timeout_ms for the work queued on s (0: look once). *done = false when it is still running at
// the deadline; the work is left queued and a later wait can pick it up.
inline cudaError_t wait_stream_for(cudaStream_t s, int64_t timeout_ms, bool* done) {
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        const cudaError_t e = cudaStreamQuery(s);
        if (e == cudaSuccess) {
            *done = true;
            return cudaSuccess;
        }
        if (e != cudaErrorNotReady) return e;
        if (std::chrono::steady_clock::now() >= deadline) {
            *done = false;
            return cudaSuccess;
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

// The device address of pinned host memory (cudaHostAlloc / cudaHostRegister: mapped into the device's
// address space), or null for pageable or device memory. Kernels may read and write pinned buffers
// through it directly (over the host link), without a staging copy.
inline void* pinned_device_view(const void* p) {
    cudaPointerAttributes a{};
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Per-kernel CUDA-event timing of host-launched work (the profiled step paths): timed() brackets a launch
// with two pooled events on its stream; collect() waits for the stream and adds the elapsed times up per
// name.
class KernelTimer {
   public:
    struct Total {
        uint64_t launches = 0;
        double ms = 0.0;
    };
    template <class F>
    void timed(const char* name, cudaStream_t s, F&& f) {
        Pending p{name, take(), take()};
        cudaEventRecord(p.a, s);
        f();
        cudaEventRecord(p.b, s);
        pending_.push_back(p);
    }
    void collect(cudaStream_t s) {
        if (pending_.empty()) return;
        cudaStreamSynchronize(s);
        for (auto& p : pending_) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, p.a, p.b);
            Total& t = totals_[p.name];
            t.launches += 1;
            t.ms += ms;
            pool_.push_back(p.a);
            pool_.push_back(p.b);
        }
        pending_.clear();
    }
    void clear() { totals_.clear(); }
    // pcisph_kernel_time entries, name order; returns the number of kernels timed
    int read(pcisph_kernel_time* out, int max_entries) const {
        int n = 0;
        for (auto& kv : totals_) {
            if (out && n < max_entries) {
                std::memset(out[n].name, 0, sizeof(out[n].name));
                std::strncpy(out[n].name, kv.first.c_str(), sizeof(out[n].name) - 1);
                out[n].launches = kv.second.launches;
                out[n].total_ms = kv.second.ms;
            }
            ++n;
        }
        return n;
    }
    // destroys the events (call with the owner's device current); the timer stays usable
    void release() {
        for (auto& p : pending_) {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
        for (auto e : pool_) cudaEventDestroy(e);
        pending_.clear();
        pool_.clear();
    }
    ~KernelTimer() { release(); }

   private:
    struct Pending {
        std::string name;
        cudaEvent_t a, b;
    };
    cudaEvent_t take() {
        if (!pool_.empty()) {
            cudaEvent_t e = pool_.back();
            pool_.pop_back();
            return e;
        }
        cudaEvent_t e;
        cudaEventCreate(&e);
        return e;
    }
    std::map<std::string, Total> totals_;
    std::vector<Pending> pending_;
    std::vector<cudaEvent_t> pool_;
};

// Fluid.cpp:125-133
inline uint32_t sort_bit_count_ref(uint32_t elements) {
    uint32_t max_value = 0;
    for (int i = 0; i < 32; i++) {
        max_value = (max_value << 1) | 1u;
        if (max_value >= elements - 1u) return (uint32_t)(i + 1);
    }
    return 32u;
}

// Bits needed for keys < bucket_count.
inline int key_bits(uint32_t bucket_count) {
    int b = 1;
    while (b < 32 && (1ull << b) < (unsigned long long)bucket_count) ++b;
    return b;
}

// update_deduced_attributes (Fluid.cpp:377-443): the same expressions, so the same floats.
inline void derive(pcisph_sim_params* p) {
    p->kernel_radius = 4.f * p->particle_radius;
    p->kernel_radius2 = std::pow(p->kernel_radius, 2.f);
    p->particle_mass = (float)((double)p->rest_density / std::pow((double)(1.f / (2.f * p->particle_radius)), 3.0));
    p->bucket_count = p->fluid_count / 2;
    p->bucket_count -= p->bucket_count % 64;
    p->bucket_count = std::max(64u, p->bucket_count);
    p->cell_size = p->kernel_radius;
    p->poly6_normalization = 315.f / (64.f * kPi * std::pow(p->kernel_radius, 9.f));
    p->poly6_d1_normalization = -945.f / (32.f * kPi * std::pow(p->kernel_radius, 9.f));
    p->viscosity_d2_normalization = 45.f / (kPi * std::pow(p->kernel_radius, 6.0f));
    p->spiky_d1_normalization = -45.f / (kPi * std::pow(p->kernel_radius, 6.0f));
    p->surface_tension_normalization = 32.f / (kPi * std::pow(p->kernel_radius, 9.f));
    p->surface_tension_term = std::pow(p->kernel_radius, 6.f) / 64.f;
    const float particle_size = 2.f * p->particle_radius;
    const float beta = p->delta_t * p->delta_t * p->particle_mass * p->particle_mass * 2.f /
                       (p->rest_density * p->rest_density);
    float sum[3] = {0.f, 0.f, 0.f}, sum_sq = 0.f;
    const float lim = p->kernel_radius + particle_size;
    for (float z = -p->kernel_radius - particle_size; z <= lim; z += 2.f * p->particle_radius)
        for (float y = -p->kernel_radius - particle_size; y <= lim; y += 2.f * p->particle_radius)
            for (float x = -p->kernel_radius - particle_size; x <= lim; x += 2.f * p->particle_radius) {
                const float r = std::sqrt(x * x + y * y + z * z);
                const float r2 = r * r;
                if (r2 < p->kernel_radius2) {
                    const float f = (float)((double)p->poly6_d1_normalization *
                                            std::pow((double)(p->kernel_radius2 - r2), 2.0));
                    const float v[3] = {-f * x, -f * y, -f * z};
                    for (int i = 0; i < 3; i++) {
                        sum[i] += v[i];
                        sum_sq += v[i] * v[i];
                    }
                }
            }
    float sum_dot = 0.f;
    for (int i = 0; i < 3; i++) sum_dot += sum[i] * sum[i];
    p->density_variation_scaling_factor = -1.f / (beta * (-sum_dot - sum_sq));
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

struct DeviceBlock {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 256));
        if (e == cudaSuccess) cap = std::max<size_t>(bytes, 256);
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

struct Carver {
    unsigned char* base;
    size_t off = 0;
    template <class T>
    T* take(size_t count) {
        T* r = reinterpret_cast<T*>(base + off);
        off += align256(count * sizeof(T));
        return r;
    }
};

// Kernel parameters of one scene from its reference parameters and step options.
inline void make_devparams(const pcisph_sim_params& p, int min_iters, int max_iters, int walls, const float* box_lo,
                           const float* box_hi, float restitution, float threshold, float list_skin,
                           uint32_t bucket_base, DevParams* d, uint32_t list_cap = kListCap,
                           int adaptive_skin = 0) {
    *d = DevParams{};
    d->particle_mass = p.particle_mass;
    d->rest_density = p.rest_density;
    d->h = p.kernel_radius;
    d->h2 = p.kernel_radius2;
    d->cell_size = p.cell_size;
    d->poly6_norm = p.poly6_normalization;
    d->poly6_d1_norm = p.poly6_d1_normalization;
    d->visc_d2_norm = p.viscosity_d2_normalization;
    d->spiky_d1_norm = p.spiky_d1_normalization;
    d->st_coeff = p.surface_tension_coefficient;
    d->st_term = p.surface_tension_term;
    d->st_norm = p.surface_tension_normalization;
    d->viscosity = p.viscosity_constant;
    d->gravity = p.gravity;
    d->dt = p.delta_t;
    d->delta = p.density_variation_scaling_factor;
    d->fluid_count = p.fluid_count;
    d->boundary_count = p.boundary_count;
    d->bucket_count = p.bucket_count;
    magic_for(p.bucket_count, &d->bk_magic, &d->bk_shift);
    d->bucket_base = bucket_base;
    d->list_cap = list_cap;
    d->near_cap = kNearCap;
    d->bnd_cap = kBoundaryListCap;
    d->bfl_cap = kBoundaryFluidCap;
    d->near_r2 = p.kernel_radius2 * 1.0001f;
    set_list_skin(d, list_skin);
    d->adaptive_skin = adaptive_skin;
    d->skin_outrun_ratio = kSkinOutrunRatio;
    for (int k = 0; k < kSkinLevels; ++k) d->skin_half[k] = 0.5f * p.kernel_radius * skin_level_value(k);
    d->min_iters = min_iters;
    d->max_iters = max_iters;
    d->walls = walls;
    for (int a = 0; a < 3; a++) {
        d->box_lo[a] = box_lo[a];
        d->box_hi[a] = box_hi[a];
    }
    d->restitution = restitution;
    d->threshold = threshold;
}

}  // namespace host
}  // namespace pcisph
