/*
 * pcisph_oracle.cpp -- CPU restatement of the reference PCISPH time step.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker for the CUDA path and the
 * timed CPU baseline ("port"); only tests/, __graft_entry__.smoke() and the
 * cpu-baseline leg of bench.py load it. The product never links or calls it.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks every function here
 * against golden vectors produced by the reference's own kernels compiled on
 * the host (oracle/build_ref.sh -> oracle/_ref, tests/golden/make_golden.py).
 *
 * What it restates (file:line in the reference, PCISPH/...):
 *   or_derive_params       src/sim/Fluid.cpp:377-443  (update_deduced_attributes)
 *   or_sort_bit_count      src/sim/Fluid.cpp:125-133
 *   or_hash_key/cell       data/kernels/grid_utils.cl:9-19
 *   neighbour walk         data/kernels/grid_utils.cl:65-79 (method 1: 27 hashed
 *                          buckets, x fastest, no duplicate-bucket removal)
 *   or_initialize          data/kernels/sort_utils.cl:12-23
 *   or_counting_sort       the clogs contract (stable key/value sort,
 *                          libs/clogs/include/clogs/radixsort.h:176-185)
 *   or_reorder             data/kernels/sort_utils.cl:25-78
 *   smoothing kernels      data/kernels/pcisph.cl:8-61
 *   or_update_density      data/kernels/pcisph.cl:65-92
 *   or_update_normal       data/kernels/pcisph.cl:94-112
 *   or_force_init          data/kernels/pcisph.cl:121-173
 *   or_advance             data/kernels/pcisph.cl:175-193
 *   or_boundary_self_density data/kernels/pcisph.cl:195-210
 *   or_update_pressure     data/kernels/pcisph.cl:212-263
 *   or_pressure_force      data/kernels/pcisph.cl:265-300
 *   or_step_f32/_f64       src/sim/Fluid.cpp:108-327 (step order, convergence
 *                          test at :250-251, :284-306)
 *
 * Arithmetic follows the reference expression by expression (same operand
 * order, IEEE float, no contraction: built with -ffp-contract=off), so the FP32
 * path reproduces the reference kernels bit for bit on the same inputs. The
 * FP64 instantiation runs the same step in double; cell keys and the sorted
 * permutation always come from the FP32 positions, as in the FP32 step.
 *
 * Extensions that the reference does not have (applied identically on the GPU):
 *   - walls: after integration each axis is clamped to [lo, hi]; a clamped
 *     velocity component that points out of the box is reflected and scaled by
 *     the restitution coefficient.
 *   - min/max iteration counts (reference: 3 and 7) and a fixed count for
 *     parity runs.
 *   - boundary_self_density: 0 leaves the boundary-boundary predicted density at
 *     zero (the reference never launches that kernel, Fluid.cpp:167-171);
 *     1 computes it.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <climits>
#include <vector>

#include <omp.h>

typedef uint32_t u32;

/* Mirror of Simulation_Params (data/kernels/Simulation_Params.h:18-44): 20 x 4 B. */
struct OrParams {
    float particle_radius;
    float particle_mass;
    float rest_density;
    u32 boundary_count;
    u32 fluid_count;
    float kernel_radius;
    float kernel_radius2;
    u32 bucket_count;
    float cell_size;
    float poly6_normalization;
    float poly6_d1_normalization;
    float viscosity_d2_normalization;
    float spiky_d1_normalization;
    float surface_tension_coefficient;
    float surface_tension_term;
    float surface_tension_normalization;
    float viscosity_constant;
    float gravity;
    float delta_t;
    float density_variation_scaling_factor;
};
static_assert(sizeof(OrParams) == 80, "Simulation_Params is 80 bytes");

struct OrOptions {
    float threshold;            /* density_variation_threshold (scenes.cpp:224: 0.01) */
    int min_iters;              /* reference: 3 (checks from i >= 2, Fluid.cpp:250, :284) */
    int max_iters;              /* reference: 7 (Fluid.cpp:251) */
    int walls;                  /* 0: reference (none), 1: reflecting box */
    float box_lo[3];
    float box_hi[3];
    float restitution;
    int boundary_self_density;  /* 0 or 1, see header */
};

static const float OR_PI = 3.14159265358979323846f; /* utils/constants.h:4 */

/* ------------------------------------------------------------------ params */

extern "C" u32 or_sort_bit_count(u32 elements) {
    u32 max_value = 0;
    for (int i = 0; i < 32; i++) {
        max_value = (max_value << 1) | 1u;
        if (max_value >= elements - 1u) return (u32)(i + 1);
    }
    return 32u;
}

/* Fluid.cpp:377-443. The std::pow calls keep their C++11 overloads: pow(float,
 * float) is float, pow(float, int) is promoted to double. */
extern "C" void or_derive_params(float particle_radius, float rest_density, u32 fluid_count, u32 boundary_count,
                                 float delta_t, float gravity, float viscosity, float surface_tension, OrParams* p) {
    std::memset(p, 0, sizeof(*p));
    p->particle_radius = particle_radius;
    p->rest_density = rest_density;
    p->fluid_count = fluid_count;
    p->boundary_count = boundary_count;
    p->delta_t = delta_t;
    p->gravity = gravity;
    p->viscosity_constant = viscosity;
    p->surface_tension_coefficient = surface_tension;

    p->kernel_radius = 4.f * p->particle_radius;
    p->kernel_radius2 = std::pow(p->kernel_radius, 2.f);
    p->particle_mass = (float)((double)p->rest_density / std::pow((double)(1.f / (2.f * p->particle_radius)), 3.0));
    p->bucket_count = p->fluid_count / 2;
    p->bucket_count -= p->bucket_count % 64;
    p->bucket_count = std::max(64u, p->bucket_count);
    p->cell_size = p->kernel_radius;
    p->poly6_normalization = 315.f / (64.f * OR_PI * std::pow(p->kernel_radius, 9.f));
    p->poly6_d1_normalization = -945.f / (32.f * OR_PI * std::pow(p->kernel_radius, 9.f));
    p->viscosity_d2_normalization = 45.f / (OR_PI * std::pow(p->kernel_radius, 6.0f));
    p->spiky_d1_normalization = -45.f / (OR_PI * std::pow(p->kernel_radius, 6.0f));
    p->surface_tension_normalization = 32.f / (OR_PI * std::pow(p->kernel_radius, 9.f));
    p->surface_tension_term = std::pow(p->kernel_radius, 6.f) / 64.f;

    const float particle_size = 2.f * p->particle_radius;
    const float beta = p->delta_t * p->delta_t * p->particle_mass * p->particle_mass * 2.f /
                       (p->rest_density * p->rest_density);
    float sum[3] = {0.f, 0.f, 0.f};
    float sum_sq = 0.f;
    const float lim = p->kernel_radius + particle_size;
    for (float z = -p->kernel_radius - particle_size; z <= lim; z += 2.f * p->particle_radius) {
        for (float y = -p->kernel_radius - particle_size; y <= lim; y += 2.f * p->particle_radius) {
            for (float x = -p->kernel_radius - particle_size; x <= lim; x += 2.f * p->particle_radius) {
                float r = std::sqrt(x * x + y * y + z * z);
                float r2 = r * r;
                if (r2 < p->kernel_radius2) {
                    float factor = (float)((double)p->poly6_d1_normalization *
                                           std::pow((double)(p->kernel_radius2 - r2), 2.0));
                    float v[3] = {-factor * x, -factor * y, -factor * z};
                    for (int i = 0; i < 3; i++) {
                        sum[i] += v[i];
                        sum_sq += v[i] * v[i];
                    }
                }
            }
        }
    }
    float sum_dot = 0.f;
    for (int i = 0; i < 3; i++) sum_dot += sum[i] * sum[i];
    p->density_variation_scaling_factor = -1.f / (beta * (-sum_dot - sum_sq));
}

/* ----------------------------------------------------------------- hashing */

static inline int or_floor_sat(float v) {  /* convert_int_sat_rtn */
    if (std::isnan(v)) return 0;
    float f = std::floor(v);
    if (f >= 2147483648.0f) return INT_MAX;
    if (f < -2147483648.0f) return INT_MIN;
    return (int)f;
}

/* grid_utils.cl:12-19 in wrapping 32-bit arithmetic. */
static inline u32 or_key(u32 x, u32 y, u32 z, u32 bk) {
    u32 h = (x * 19349663u) ^ (y * 73856093u) ^ (z * 83492791u);
    u32 v = (h << 6) + (x & 63u) + 4u * (y & 63u) + 16u * (z & 63u);
    return (v & 0x7FFFFFFFu) % bk;
}

extern "C" u32 or_hash_key(int x, int y, int z, u32 bk) { return or_key((u32)x, (u32)y, (u32)z, bk); }

struct Cell { int x, y, z; };
static inline Cell or_cell(float px, float py, float pz, float cell) {  /* grid_utils.cl:9-11 */
    return Cell{or_floor_sat(px / cell), or_floor_sat(py / cell), or_floor_sat(pz / cell)};
}

extern "C" void or_cell_pos(float px, float py, float pz, float cell, int* out) {
    Cell c = or_cell(px, py, pz, cell);
    out[0] = c.x; out[1] = c.y; out[2] = c.z;
}

/* The 27 bucket keys around a cell in walk order (grid_utils.cl:68-69). */
static inline void or_neighbour_keys(const Cell& c, u32 bk, u32 keys[27]) {
    for (int i = 0; i < 27; i++) {
        int dx = (i % 3) - 1, dy = ((i / 3) % 3) - 1, dz = ((i / 9) % 3) - 1;
        keys[i] = or_key((u32)c.x + (u32)dx, (u32)c.y + (u32)dy, (u32)c.z + (u32)dz, bk);
    }
}

template <typename F>
static inline void or_foreach(const u32* offsets, const u32 keys[27], F&& body) {
    for (int i = 0; i < 27; i++) {
        u32 s = offsets[2 * keys[i]], e = offsets[2 * keys[i] + 1];
        for (u32 j = s; j < e; j++) body(j);
    }
}

/* sort_utils.cl:12-23 */
extern "C" void or_initialize(const OrParams* p, u32 n, const float* pos, u32* keys, u32* src) {
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; i++) {
        Cell c = or_cell(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], p->cell_size);
        keys[i] = or_key((u32)c.x, (u32)c.y, (u32)c.z, p->bucket_count);
        src[i] = (u32)i;
    }
}

/* Stable counting sort of (key, value) for keys < bk: the clogs contract. */
extern "C" void or_counting_sort(u32* keys, u32* vals, u32 n, u32 bk) {
    std::vector<u32> count((size_t)bk + 1, 0u), k(n), v(n);
    for (u32 i = 0; i < n; i++) count[keys[i] + 1]++;
    for (u32 b = 0; b < bk; b++) count[b + 1] += count[b];
    for (u32 i = 0; i < n; i++) {
        u32 d = count[keys[i]]++;
        k[d] = keys[i];
        v[d] = vals[i];
    }
    std::memcpy(keys, k.data(), (size_t)n * 4);
    std::memcpy(vals, v.data(), (size_t)n * 4);
}

/* sort_utils.cl:7-10 then :25-78. cell_offsets (2*bk) is cleared here. in_vel/out_vel may be NULL. */
extern "C" void or_reorder(u32 n, u32 bk, const u32* keys, const u32* src, const float* in_pos, const float* in_vel,
                           float* out_pos, float* out_vel, u32* cell_offsets) {
    std::memset(cell_offsets, 0, (size_t)bk * 2 * sizeof(u32));
#pragma omp parallel for schedule(static)
    for (long long d = 0; d < (long long)n; d++) {
        u32 s = src[d];
        for (int a = 0; a < 3; a++) out_pos[3 * d + a] = in_pos[3 * (size_t)s + a];
        if (in_vel)
            for (int a = 0; a < 3; a++) out_vel[3 * d + a] = in_vel[3 * (size_t)s + a];
        u32 key = keys[d];
        if (d == 0 || key != keys[d - 1]) cell_offsets[2 * key] = (u32)d;
        if (d == (long long)n - 1 || key != keys[d + 1]) cell_offsets[2 * key + 1] = (u32)d + 1;
    }
}

/* -------------------------------------------------------- smoothing kernels */

template <typename T> struct V3 {
    T x, y, z;
};
template <typename T> static inline V3<T> ld3(const T* a, size_t i) { return V3<T>{a[3 * i], a[3 * i + 1], a[3 * i + 2]}; }
template <typename T> static inline void st3(T* a, size_t i, V3<T> v) { a[3 * i] = v.x; a[3 * i + 1] = v.y; a[3 * i + 2] = v.z; }
template <typename T> static inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T> static inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T> static inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename T> static inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T> static inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <typename T> static inline T dot3(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

template <typename T> static inline T k_poly6(T r2, T h2) {  /* pcisph.cl:8-16 */
    if (r2 > h2) return T(0);
    T dr = h2 - r2;
    return dr * dr * dr;
}
template <typename T> static inline V3<T> k_poly6_d1(V3<T> d, T h2) {  /* pcisph.cl:18-26 */
    T r2 = dot3(d, d);
    if (r2 > h2) return V3<T>{0, 0, 0};
    return (r2 - h2) * (r2 - h2) * d;
}
template <typename T> static inline V3<T> k_spiky_d1(V3<T> d, T h) {  /* pcisph.cl:28-37 */
    T r = std::sqrt(dot3(d, d));
    if (r > h || r < T(0.0001f)) return V3<T>{0, 0, 0};
    T dr = h - r;
    return d * dr * dr / r;
}
template <typename T> static inline T k_visc_d2(T r, T h) { return r > h ? T(0) : h - r; }  /* pcisph.cl:39-46 */
template <typename T> static inline T k_surface_tension(T r, T h, T st_term) {  /* pcisph.cl:48-61 */
    if ((double)r <= 0.5 * (double)h) {
        T t1 = h - r;
        T t2 = (t1 * t1 * t1) * (r * r * r);
        return T(2) * t2 - st_term;
    } else if (r <= h) {
        T t1 = h - r;
        return (t1 * t1 * t1) * (r * r * r);
    }
    return T(0);
}

/* ------------------------------------------------------------ step kernels */

/* Cell keys of a particle come from its FP32 position in every precision. */
template <typename T> static inline Cell cell_of(const T* pos, size_t i, float cell) {
    return or_cell((float)pos[3 * i], (float)pos[3 * i + 1], (float)pos[3 * i + 2], cell);
}

/* pcisph.cl:65-92. b_off may be NULL when there are no boundary particles. */
template <typename T>
static void density(const OrParams* p, const u32* b_off, const T* b_pos, const u32* f_off, const T* f_pos, T* rho) {
    const T h2 = (T)p->kernel_radius2;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)p->fluid_count; i++) {
        V3<T> x = ld3(f_pos, i);
        u32 keys[27];
        or_neighbour_keys(cell_of(f_pos, i, p->cell_size), p->bucket_count, keys);
        T acc = 0;
        if (b_off && p->boundary_count)
            or_foreach(b_off, keys, [&](u32 j) { V3<T> d = x - ld3(b_pos, j); acc += k_poly6(dot3(d, d), h2); });
        or_foreach(f_off, keys, [&](u32 j) { V3<T> d = x - ld3(f_pos, j); acc += k_poly6(dot3(d, d), h2); });
        acc *= (T)p->particle_mass * (T)p->poly6_normalization;
        rho[i] = acc;
    }
}

/* pcisph.cl:94-112 */
template <typename T>
static void normal(const OrParams* p, const u32* f_off, const T* f_pos, const T* rho, T* nrm) {
    const T h2 = (T)p->kernel_radius2;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)p->fluid_count; i++) {
        V3<T> x = ld3(f_pos, i);
        u32 keys[27];
        or_neighbour_keys(cell_of(f_pos, i, p->cell_size), p->bucket_count, keys);
        V3<T> n{0, 0, 0};
        or_foreach(f_off, keys, [&](u32 j) { n = n + k_poly6_d1(x - ld3(f_pos, j), h2) / rho[j]; });
        n = n * ((T)p->kernel_radius * (T)p->particle_mass * (T)p->poly6_d1_normalization);
        st3(nrm, i, n);
    }
}

/* pcisph.cl:121-173 (also zeroes pressure and pressure force) */
template <typename T>
static void force_init(const OrParams* p, const u32* f_off, const T* pos, const T* nrm, const T* rho, const T* vel,
                       T* f_other, T* press, T* f_press) {
    const T h = (T)p->kernel_radius, rho0 = (T)p->rest_density;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)p->fluid_count; i++) {
        V3<T> x = ld3(pos, i), v = ld3(vel, i), n = ld3(nrm, i);
        T ri = rho[i];
        u32 keys[27];
        or_neighbour_keys(cell_of(pos, i, p->cell_size), p->bucket_count, keys);
        V3<T> visc{0, 0, 0}, coh{0, 0, 0}, curv{0, 0, 0};
        or_foreach(f_off, keys, [&](u32 j) {
            V3<T> xj = ld3(pos, j), vj = ld3(vel, j), nj = ld3(nrm, j);
            T rj = rho[j];
            V3<T> dx = x - xj;
            T dist = std::sqrt(dot3(dx, dx));
            if (rj > T(0.0001f)) visc = visc + (vj - v) * (k_visc_d2(dist, h) / rj);
            if (dist > T(0.0001f) && dist < h) {
                T corr = T(2) * rho0 / (ri + rj);
                T stk = k_surface_tension(dist, h, (T)p->surface_tension_term);
                V3<T> dir = (x - xj) / dist;
                coh = coh + corr * stk * dir;
                curv = curv + corr * (n - nj);
            }
        });
        visc = visc * ((T)p->viscosity_constant * (T)p->particle_mass * (T)p->viscosity_d2_normalization);
        coh = coh * (-(T)p->surface_tension_coefficient * (T)p->particle_mass * (T)p->particle_mass *
                     (T)p->surface_tension_normalization);
        curv = curv * (-(T)p->surface_tension_coefficient * (T)p->particle_mass);
        V3<T> st = coh + curv;
        V3<T> g{0, (T)p->particle_mass * (T)p->gravity, 0};
        st3(f_other, i, g + visc + st);
        press[i] = 0;
        st3(f_press, i, V3<T>{0, 0, 0});
    }
}

/* Walls (extension, see header). */
template <typename T> static inline void apply_walls(const OrOptions* o, V3<T>& x, V3<T>& v) {
    T* xs[3] = {&x.x, &x.y, &x.z};
    T* vs[3] = {&v.x, &v.y, &v.z};
    for (int a = 0; a < 3; a++) {
        T lo = (T)o->box_lo[a], hi = (T)o->box_hi[a], e = (T)o->restitution;
        if (*xs[a] < lo) {
            *xs[a] = lo;
            if (*vs[a] < T(0)) *vs[a] = -e * *vs[a];
        } else if (*xs[a] > hi) {
            *xs[a] = hi;
            if (*vs[a] > T(0)) *vs[a] = -e * *vs[a];
        }
    }
}

/* pcisph.cl:175-193. new_vel NULL = predict; walls only when integrating with o->walls. */
template <typename T>
static void advance(const OrParams* p, const OrOptions* o, const T* pos, const T* vel, const T* f_other,
                    const T* f_press, T* new_pos, T* new_vel) {
    const T m = (T)p->particle_mass, dt = (T)p->delta_t;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)p->fluid_count; i++) {
        V3<T> x = ld3(pos, i), v = ld3(vel, i);
        V3<T> f = ld3(f_other, i) + ld3(f_press, i);
        V3<T> a = f / m;
        v = v + a * dt;
        x = x + v * dt;
        if (new_vel && o && o->walls) apply_walls(o, x, v);
        st3(new_pos, i, x);
        if (new_vel) st3(new_vel, i, v);
    }
}

/* pcisph.cl:195-210: raw sum, without the m*K factor. */
template <typename T>
static void boundary_self_density(const OrParams* p, const u32* b_off, const T* b_pos, T* out) {
    const T h2 = (T)p->kernel_radius2;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)p->boundary_count; i++) {
        V3<T> x = ld3(b_pos, i);
        u32 keys[27];
        or_neighbour_keys(cell_of(b_pos, i, p->cell_size), p->bucket_count, keys);
        T acc = 0;
        or_foreach(b_off, keys, [&](u32 j) { V3<T> d = x - ld3(b_pos, j); acc += k_poly6(dot3(d, d), h2); });
        out[i] = acc;
    }
}

/* pcisph.cl:212-263. Cells are searched around the current position, distances
 * taken between predicted positions. err may be NULL. */
template <typename T>
static void pressure(const OrParams* p, int boundary_update, const u32* b_off, const T* b_pos, const T* b_init,
                     const u32* f_off, const T* f_pos, const T* f_pred, T* err, T* out_press) {
    const T h2 = (T)p->kernel_radius2;
    const long long count = boundary_update ? p->boundary_count : p->fluid_count;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < count; i++) {
        V3<T> x, xp;
        Cell c;
        if (boundary_update) {
            x = ld3(b_pos, i);
            xp = x;
            c = cell_of(b_pos, i, p->cell_size);
        } else {
            x = ld3(f_pos, i);
            xp = ld3(f_pred, i);
            c = cell_of(f_pos, i, p->cell_size);
        }
        u32 keys[27];
        or_neighbour_keys(c, p->bucket_count, keys);
        T acc = 0;
        if (boundary_update) {
            acc += b_init ? b_init[i] : T(0);
        } else if (b_off && p->boundary_count) {
            or_foreach(b_off, keys, [&](u32 j) { V3<T> d = xp - ld3(b_pos, j); acc += k_poly6(dot3(d, d), h2); });
        }
        or_foreach(f_off, keys, [&](u32 j) { V3<T> d = xp - ld3(f_pred, j); acc += k_poly6(dot3(d, d), h2); });
        acc *= (T)p->particle_mass * (T)p->poly6_normalization;
        T dv = acc - (T)p->rest_density;
        dv = T(0) < dv ? dv : T(0);  /* OpenCL max(0, x) */
        if (err) err[i] = dv;
        if (dv == T(0)) continue;
        out_press[i] += dv * (T)p->density_variation_scaling_factor;
    }
}

/* pcisph.cl:265-300 */
template <typename T>
static void pressure_force(const OrParams* p, const u32* b_off, const T* b_pos, const T* b_press, const u32* f_off,
                           const T* f_pos, const T* rho, const T* press, T* f_press) {
    const T h = (T)p->kernel_radius, rho0 = (T)p->rest_density;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)p->fluid_count; i++) {
        V3<T> x = ld3(f_pos, i);
        T self_factor = press[i] / (rho[i] * rho[i]);
        u32 keys[27];
        or_neighbour_keys(cell_of(f_pos, i, p->cell_size), p->bucket_count, keys);
        V3<T> f{0, 0, 0};
        if (b_off && p->boundary_count)
            or_foreach(b_off, keys, [&](u32 j) {
                T other = b_press[j] / (rho0 * rho0);
                f = f + k_spiky_d1(x - ld3(b_pos, j), h) * (self_factor + other);
            });
        or_foreach(f_off, keys, [&](u32 j) {
            T other = press[j] / (rho[j] * rho[j]);
            f = f + k_spiky_d1(x - ld3(f_pos, j), h) * (self_factor + other);
        });
        f = f * (-(T)p->spiky_d1_normalization * (T)p->particle_mass * (T)p->particle_mass);
        st3(f_press, i, f);
    }
}

/* ----------------------------------------------------------- FP32 exports */

extern "C" {
int or_sizeof_params(void) { return (int)sizeof(OrParams); }
int or_sizeof_options(void) { return (int)sizeof(OrOptions); }
// The OpenMP threads a parallel region of this library runs on (the CPU baseline reports them).
int or_num_threads(void) { return omp_get_max_threads(); }
void or_update_density(const OrParams* p, const u32* b_off, const float* b_pos, const u32* f_off, const float* f_pos,
                       float* rho) { density<float>(p, b_off, b_pos, f_off, f_pos, rho); }
void or_update_normal(const OrParams* p, const u32* f_off, const float* f_pos, const float* rho, float* nrm) {
    normal<float>(p, f_off, f_pos, rho, nrm);
}
void or_force_init(const OrParams* p, const u32* f_off, const float* pos, const float* nrm, const float* rho,
                   const float* vel, float* f_other, float* press, float* f_press) {
    force_init<float>(p, f_off, pos, nrm, rho, vel, f_other, press, f_press);
}
void or_advance(const OrParams* p, const OrOptions* o, const float* pos, const float* vel, const float* f_other,
                const float* f_press, float* new_pos, float* new_vel) {
    advance<float>(p, o, pos, vel, f_other, f_press, new_pos, new_vel);
}
void or_boundary_self_density(const OrParams* p, const u32* b_off, const float* b_pos, float* out) {
    boundary_self_density<float>(p, b_off, b_pos, out);
}
void or_update_pressure(const OrParams* p, int boundary_update, const u32* b_off, const float* b_pos,
                        const float* b_init, const u32* f_off, const float* f_pos, const float* f_pred, float* err,
                        float* out_press) {
    pressure<float>(p, boundary_update, b_off, b_pos, b_init, f_off, f_pos, f_pred, err, out_press);
}
void or_pressure_force(const OrParams* p, const u32* b_off, const float* b_pos, const float* b_press, const u32* f_off,
                       const float* f_pos, const float* rho, const float* press, float* f_press) {
    pressure_force<float>(p, b_off, b_pos, b_press, f_off, f_pos, rho, press, f_press);
}
}

/* -------------------------------------------------------------- full step */

/*
 * State of one scene. Vectors are packed xyz (the reference layout, 12 B per
 * particle in FP32). f_pos/f_vel are read and written; after the step every
 * fluid array is in this step's sorted order, as in the reference. The boundary
 * arrays are sorted in place when boundary_sort is set (and b_init filled);
 * otherwise they must already be sorted with b_off filled.
 */
template <typename T> struct OrState {
    T *f_pos, *f_vel, *f_normal, *f_pred, *f_rho, *f_other, *f_press, *f_fpress, *f_err;
    T *b_pos, *b_press, *b_init;
    u32 *f_keys, *f_src, *f_off, *b_keys, *b_src, *b_off;
};

struct OrStats {
    int iterations;
    float max_err;      /* max density variation of the last iteration (kg/m^3) */
    int converged;      /* max_err / rho0 < threshold reached within max_iters */
};

template <typename T>
static int step(const OrParams* p, const OrOptions* o, OrState<T>* s, int boundary_sort, OrStats* st) {
    const u32 N = p->fluid_count, B = p->boundary_count, bk = p->bucket_count;
    if (N == 0) return 0;
    std::vector<float> kp;  /* FP32 copy of positions for keys */
    if (boundary_sort && B > 0) {
        kp.resize(3 * (size_t)B);
        for (size_t i = 0; i < kp.size(); i++) kp[i] = (float)s->b_pos[i];
        or_initialize(p, B, kp.data(), s->b_keys, s->b_src);
        or_counting_sort(s->b_keys, s->b_src, B, bk);
        std::vector<T> tmp(s->b_pos, s->b_pos + 3 * (size_t)B);
        std::memset(s->b_off, 0, (size_t)bk * 2 * sizeof(u32));
        for (u32 d = 0; d < B; d++) {
            u32 src = s->b_src[d];
            for (int a = 0; a < 3; a++) s->b_pos[3 * (size_t)d + a] = tmp[3 * (size_t)src + a];
            u32 key = s->b_keys[d];
            if (d == 0 || key != s->b_keys[d - 1]) s->b_off[2 * key] = d;
            if (d == B - 1 || key != s->b_keys[d + 1]) s->b_off[2 * key + 1] = d + 1;
        }
        if (o->boundary_self_density) boundary_self_density<T>(p, s->b_off, s->b_pos, s->b_init);
        else std::memset(s->b_init, 0, (size_t)B * sizeof(T));
    }
    /* sort and reorder the fluid (Fluid.cpp:176-207) */
    kp.resize(3 * (size_t)N);
    for (size_t i = 0; i < kp.size(); i++) kp[i] = (float)s->f_pos[i];
    or_initialize(p, N, kp.data(), s->f_keys, s->f_src);
    or_counting_sort(s->f_keys, s->f_src, N, bk);
    {
        std::vector<T> tp(s->f_pos, s->f_pos + 3 * (size_t)N), tv(s->f_vel, s->f_vel + 3 * (size_t)N);
        std::memset(s->f_off, 0, (size_t)bk * 2 * sizeof(u32));
#pragma omp parallel for schedule(static)
        for (long long d = 0; d < (long long)N; d++) {
            u32 src = s->f_src[d];
            for (int a = 0; a < 3; a++) {
                s->f_pos[3 * d + a] = tp[3 * (size_t)src + a];
                s->f_vel[3 * d + a] = tv[3 * (size_t)src + a];
            }
            u32 key = s->f_keys[d];
            if (d == 0 || key != s->f_keys[d - 1]) s->f_off[2 * key] = (u32)d;
            if (d == (long long)N - 1 || key != s->f_keys[d + 1]) s->f_off[2 * key + 1] = (u32)d + 1;
        }
    }
    const u32* boff = B ? s->b_off : nullptr;
    density<T>(p, boff, s->b_pos, s->f_off, s->f_pos, s->f_rho);
    normal<T>(p, s->f_off, s->f_pos, s->f_rho, s->f_normal);
    if (B > 0) std::fill(s->b_press, s->b_press + B, T(0));
    force_init<T>(p, s->f_off, s->f_pos, s->f_normal, s->f_rho, s->f_vel, s->f_other, s->f_press, s->f_fpress);

    int iters = 0;
    T max_err = 0;
    bool converged = false;
    for (int i = 0; i < o->max_iters; i++) {
        advance<T>(p, nullptr, s->f_pos, s->f_vel, s->f_other, s->f_fpress, s->f_pred, nullptr);
        if (B > 0) pressure<T>(p, 1, boff, s->b_pos, s->b_init, s->f_off, s->f_pos, s->f_pred, nullptr, s->b_press);
        pressure<T>(p, 0, boff, s->b_pos, s->b_init, s->f_off, s->f_pos, s->f_pred, s->f_err, s->f_press);
        pressure_force<T>(p, boff, s->b_pos, s->b_press, s->f_off, s->f_pos, s->f_rho, s->f_press, s->f_fpress);
        iters = i + 1;
        max_err = *std::max_element(s->f_err, s->f_err + N);
        converged = (float)max_err / p->rest_density < o->threshold;
        if (iters >= o->min_iters && converged) break;
    }
    advance<T>(p, o, s->f_pos, s->f_vel, s->f_other, s->f_fpress, s->f_pos, s->f_vel);
    if (st) {
        st->iterations = iters;
        st->max_err = (float)max_err;
        st->converged = converged ? 1 : 0;
    }
    return iters;
}

extern "C" {
int or_step_f32(const OrParams* p, const OrOptions* o, OrState<float>* s, int boundary_sort, OrStats* st) {
    return step<float>(p, o, s, boundary_sort, st);
}
int or_step_f64(const OrParams* p, const OrOptions* o, OrState<double>* s, int boundary_sort, OrStats* st) {
    return step<double>(p, o, s, boundary_sort, st);
}
// pcisph.cl:121-173 in FP64 on the given (FP32-valued) inputs: the rerun that settles pairs at r = h
void or_force_init_f64(const OrParams* p, const u32* f_off, const double* pos, const double* nrm, const double* rho,
                       const double* vel, double* f_other, double* press, double* f_press) {
    force_init<double>(p, f_off, pos, nrm, rho, vel, f_other, press, f_press);
}
}
