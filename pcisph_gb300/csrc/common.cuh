// common.cuh -- device-side vocabulary shared by the PCISPH kernels.
//
// Hashing is bit-exact with the reference (PCISPH/data/kernels/grid_utils.cl:9-19):
//   cell = floor_sat(pos / cell_size)  (IEEE division, NaN -> 0, saturating)
//   key  = ((((x*19349663) ^ (y*73856093) ^ (z*83492791)) << 6)
//           + (x&63) + 4(y&63) + 16(z&63)) & 0x7FFFFFFF) % bucket_count
// in wrapping 32-bit arithmetic. The modulo uses a precomputed multiplier
// (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, Thm 4.2): for n < 2^31 and l = ceil(log2 d),
// m = ceil(2^(31+l) / d) < 2^32 gives floor(n/d) = umulhi(n, m) >> (l-1).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pcisph {

// Everything a step kernel needs, passed by value (lives in the constant bank).
struct DevParams {
    // reference fields (Simulation_Params)
    float particle_mass, rest_density, h, h2, cell_size;
    float poly6_norm, poly6_d1_norm, visc_d2_norm, spiky_d1_norm;
    float st_coeff, st_term, st_norm, viscosity, gravity, dt, delta;
    uint32_t fluid_count, boundary_count, bucket_count;
    // modulo by bucket_count
    uint32_t bk_magic, bk_shift;
    // first entry of this scene's buckets in a cell table shared by several scenes (0 for one scene)
    uint32_t bucket_base;
    // neighbour lists (kernel_variant 2): capacity per particle, radius h (1 + skin) and its square
    uint32_t list_cap;
    uint32_t near_cap;  // entries of the within-h list
    uint32_t bnd_cap;   // entries of the boundary list (boundary particles within r_list)
    uint32_t bfl_cap;   // entries of a boundary particle's fluid list (fluid particles within r_list)
    float near_r2;      // within-h list radius^2: h^2 (1 + 1e-4), a margin far above rounding
    float list_r, list_r2, list_half_skin;
    // per-particle skins (one scene): particle i's lists take the radius h + sh_i + skin_max_half, sh_i its own
    // half skin (twice its largest predicted displacement of the previous step, within [skin_min_half,
    // skin_max_half]); a prediction past its own sh_i makes that particle walk, one past skin_max_half makes
    // its neighbourhood walk (as with one skin). 0: every particle has skin_max_half (half the list skin).
    int particle_skin;
    float skin_min_half, skin_max_half, skin_factor;
    // partner marks (one scene, list sweeps): a prediction round with at most mark_cap fast predictions lists
    // them, and a kernel stamps the particles whose pressure sweep must walk because of them; 0: off (every
    // particle near a flagged bucket walks)
    uint32_t mark_cap;
    // batched scenes with an adaptive skin: each step picks one of kSkinLevels skins from the previous
    // step's count of predictions past each level's half skin (skin_half[k])
    int adaptive_skin;
    float skin_half[3];
    uint32_t skin_outrun_ratio;  // a level qualifies if at most 1 in this many predictions outran it
    // options
    int min_iters, max_iters, walls;
    float box_lo[3], box_hi[3], restitution, threshold;
};

struct Control {
    unsigned int iter;           // iteration index within the current step
    unsigned int max_err_bits;   // float bits of the running max density variation (>= 0)
    unsigned int done;           // the loop stops after this iteration's pressure force
    unsigned int blocks_done;    // last-block counter of the reduction
    unsigned int status;         // pcisph_step_status bits of the current step
    unsigned int status_all;
    int iterations_last;
    float max_err_last;          // max variation / rest density
    unsigned long long steps;
    unsigned long long total_iters;
    unsigned int guard_iters;    // loop iterations counted by the pressure-force kernel (bounds the graph loop)
    unsigned int n_groups;       // bucket runs listed by the reorder kernel this step
    unsigned long long list_fallbacks;  // pressure sweeps in which some particle moved more than skin / 2
    unsigned long long fast_particles;  // predictions that moved more than skin / 2 (each flags its bucket)
    unsigned long long fast_at_begin;   // fast_particles when the step began: a larger count now means some
                                        // prediction of this step outran the lists
    unsigned int finished;       // batched scenes: the step is complete (no more corrective iterations)
    unsigned int any_running;    // batch control: some scene still iterates
    unsigned int skin_level;     // adaptive skin: the level of the current step
    unsigned long long over_level[3];  // adaptive skin: this step's predictions past each level's half skin
    unsigned long long unconverged_steps;  // steps that ended at max_iters with the variation above threshold
    unsigned int max_err_max_bits;         // float bits of the largest end-of-step max variation / rest density
    // partner marks (DevParams::mark_cap): fast predictions of the current round (those below mark_cap are in
    // the fast list), and the number of prediction rounds closed (round + 1 stamps the particles that walk in
    // the current round's pressure sweep, whose last block closes the round)
    unsigned long long fast_n;
    unsigned int round;
};

// Close a step after its last corrective iteration `it` (Fluid.cpp:301-306 decides the same way): status
// bit 0 when the step ended above the threshold, and the step's statistics.
__device__ __forceinline__ void close_step(Control* ctl, unsigned it, float rel, bool converged) {
    if (!converged) {
        ctl->status |= 1u;
        ctl->unconverged_steps += 1;
    }
    ctl->status_all |= ctl->status;
    ctl->iterations_last = (int)it;
    ctl->max_err_last = rel;
    // rel >= 0: its bit pattern orders like its value (a NaN variation is flagged by status bit 1)
    if (rel >= 0.f && __float_as_uint(rel) > ctl->max_err_max_bits) ctl->max_err_max_bits = __float_as_uint(rel);
    ctl->steps += 1;
    ctl->total_iters += it;
}

// List skins (units of h) an adaptive scene chooses from, smallest first.
constexpr int kSkinLevels = 3;
__host__ __device__ inline float skin_level_value(int k) { return k <= 0 ? 0.25f : k == 1 ? 0.35f : 0.5f; }

// The list radius h (1 + skin) and half the skin, less a margin for the rounding of |x_i - x_j| and
// |x* - x| (relative 1e-6 of h): a prediction within list_half_skin of x keeps every list exact.
__host__ __device__ inline void set_list_skin(DevParams* d, float skin) {
    d->list_r = d->h * (1.f + skin);
    d->list_r2 = d->list_r * d->list_r;
    d->list_half_skin = 0.5f * d->h * skin - 1e-6f * d->h;
    d->skin_max_half = 0.5f * d->h * skin;
}

// Particle k's half skin from its stored value w (the largest, skin_max_half, without per-particle skins or
// when w is 0, NaN or out of range).
__host__ __device__ inline float half_skin_of(const DevParams& P, float w) {
    return (P.particle_skin && w >= P.skin_min_half && w <= P.skin_max_half) ? w : P.skin_max_half;
}

// A prediction that moved farther than this from x is fast (its lists may miss a pair): half the skin less
// a margin for the rounding of |x* - x| and |x_i - x_j| (1e-6 h, far above it).
__host__ __device__ inline float fast_threshold(const DevParams& P, float half_skin) {
    return half_skin - 1e-6f * P.h;
}

// The list radius^2 of particle i (half skin sh_i) for fluid candidates: a pair within h at the predictions
// is within h + d_i + d_j at x, so h + sh_i + skin_max_half holds it while i moved at most sh_i and the
// candidate at most skin_max_half (a candidate past it flags its bucket). Without per-particle skins: the
// list radius h (1 + skin).
__host__ __device__ inline float particle_list_r2(const DevParams& P, float sh_i) {
    if (!P.particle_skin) return P.list_r2;
    const float r = P.h + sh_i + P.skin_max_half;
    return r * r;
}

// The same for a boundary candidate (boundary particles do not move).
__host__ __device__ inline float boundary_list_r2(const DevParams& P, float sh_i) {
    if (!P.particle_skin) return P.list_r2;
    const float r = P.h + sh_i;
    return r * r;
}

__host__ __device__ inline void magic_for(uint32_t d, uint32_t* magic, uint32_t* shift) {
    uint32_t l = 0;
    while (l < 32 && (1ull << l) < (unsigned long long)d) ++l;  // l = ceil(log2 d)
    unsigned long long m = ((1ull << (31 + l)) + d - 1) / d;     // ceil(2^(31+l)/d), d >= 2
    *magic = (uint32_t)m;
    *shift = l - 1;
}

__device__ __forceinline__ uint32_t mod_bk(uint32_t v, const DevParams& P) {
    uint32_t q = __umulhi(v, P.bk_magic) >> P.bk_shift;
    return v - q * P.bucket_count;
}

// convert_int_sat_rtn
__device__ __forceinline__ int floor_sat(float v) {
    if (v != v) return 0;
    float f = floorf(v);
    if (f >= 2147483648.0f) return 0x7FFFFFFF;
    if (f < -2147483648.0f) return (int)0x80000000;
    return (int)f;
}

struct Cell {
    uint32_t x, y, z;
};

__device__ __forceinline__ Cell cell_of(float px, float py, float pz, const DevParams& P) {
    return Cell{(uint32_t)floor_sat(__fdiv_rn(px, P.cell_size)), (uint32_t)floor_sat(__fdiv_rn(py, P.cell_size)),
                (uint32_t)floor_sat(__fdiv_rn(pz, P.cell_size))};
}

__device__ __forceinline__ uint32_t hash_key(uint32_t x, uint32_t y, uint32_t z, const DevParams& P) {
    uint32_t h = (x * 19349663u) ^ (y * 73856093u) ^ (z * 83492791u);
    uint32_t v = (h << 6) + (x & 63u) + 4u * (y & 63u) + 16u * (z & 63u);
    return mod_bk(v & 0x7FFFFFFFu, P);
}

// The ranges of the 27 neighbour buckets in the reference's walk order (grid_utils.cl:68-69: x fastest).
// body(r) is called for every bucket's [r.x, r.y); no bucket is skipped or merged.
template <class Body>
__device__ __forceinline__ void for_each_bucket(const uint2* __restrict__ cells, const Cell& c, const DevParams& P,
                                                Body&& body) {
#pragma unroll 1
    for (int dz = -1; dz <= 1; ++dz) {
        const uint32_t z = c.z + (uint32_t)dz;
        const uint32_t hz = z * 83492791u, lz = 16u * (z & 63u);
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
            const uint32_t y = c.y + (uint32_t)dy;
            const uint32_t hyz = (y * 73856093u) ^ hz, lyz = 4u * (y & 63u) + lz;
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                const uint32_t x = c.x + (uint32_t)dx;
                const uint32_t v = (((x * 19349663u) ^ hyz) << 6) + (x & 63u) + lyz;
                body(__ldg(&cells[P.bucket_base + mod_bk(v & 0x7FFFFFFFu, P)]));
            }
        }
    }
}

// The same walk with more loads in flight: load(j) -- the gather -- runs for up to 2 candidates of a
// bucket before use(j, value) consumes them in order (list builder at 1M: 668 us with 2, 672 with 1, 680
// with 4, 692 with 3, 745 with 8). Visits exactly the particles of for_each_neighbour, in the same order.
template <class Load, class Use>
__device__ __forceinline__ void for_each_neighbour_prefetched(const uint2* __restrict__ cells, const Cell& c,
                                                              const DevParams& P, Load&& load, Use&& use) {
    for_each_bucket(cells, c, P, [&](uint2 r) {
#pragma unroll 1
        for (uint32_t j = r.x; j < r.y; j += 2) {
            decltype(load(j)) o[2];
#pragma unroll
            for (int u = 0; u < 2; ++u)
                if (j + u < r.y) o[u] = load(j + u);
#pragma unroll
            for (int u = 0; u < 2; ++u)
                if (j + u < r.y) use(j + u, o[u]);
        }
    });
}

// body(j) for every particle index j of every neighbour bucket, in the walk order.
template <class Body>
__device__ __forceinline__ void for_each_neighbour(const uint2* __restrict__ cells, const Cell& c,
                                                   const DevParams& P, Body&& body) {
    for_each_bucket(cells, c, P, [&](uint2 r) {
        for (uint32_t j = r.x; j < r.y; ++j) body(j);
    });
}

// ---------------------------------------------------------------- vectors
__device__ __forceinline__ float3 f3(const float4& a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return make_float3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float4 f4(float3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// ------------------------------------------------------ fixed rounding
// A sum of products leaves the compiler a choice of which product to fuse into an FMA, and the choice can
// differ between kernels and template instantiations. These helpers fix the rounding, so every kernel
// computes the same bits for the same inputs (one scene alone or in a batch, either particle order).

// |d|^2 = dz^2 + (dy^2 + dx^2), each step rounded once
__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// F_other (pcisph.cl:161-172): (gravity + viscosity) + (cohesion + curvature), from the three neighbour
// sums and their factors
__device__ __forceinline__ float3 other_force(float m, float gravity, const float3& visc, float cv, const float3& coh,
                                              float cc, const float3& curv, float cu) {
    const float x = __fadd_rn(__fmul_rn(visc.x, cv), __fadd_rn(__fmul_rn(coh.x, cc), __fmul_rn(curv.x, cu)));
    const float y = __fadd_rn(__fadd_rn(__fmul_rn(m, gravity), __fmul_rn(visc.y, cv)),
                              __fadd_rn(__fmul_rn(coh.y, cc), __fmul_rn(curv.y, cu)));
    const float z = __fadd_rn(__fmul_rn(visc.z, cv), __fadd_rn(__fmul_rn(coh.z, cc), __fmul_rn(curv.z, cu)));
    return make_float3(x, y, z);
}

// ------------------------------------------------------ smoothing kernels (pcisph.cl:8-61)
__device__ __forceinline__ float poly6(float r2, float h2) {
    const float dr = h2 - r2;
    return r2 > h2 ? 0.f : dr * dr * dr;
}
__device__ __forceinline__ float surface_tension_kernel(float r, float h, float st_term) {
    const float t1 = h - r;
    const float t = (t1 * t1 * t1) * (r * r * r);
    if (r <= 0.5f * h) return 2.f * t - st_term;
    return r <= h ? t : 0.f;
}

}  // namespace pcisph
