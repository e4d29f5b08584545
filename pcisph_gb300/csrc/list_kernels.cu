// list_kernels.cu -- neighbour-list sweeps (kernel_variant 2).
//
// The density sweep walks the reference's 27 buckets (grid_utils.cl:65-79) once per step and records,
// per particle, every candidate j with |x_i - x_j| <= r_list = h (1 + skin), in walk order. The later
// sweeps of the step (normal, force, and the pressure and pressure-force sweeps of every corrective
// iteration) iterate that list instead of walking the buckets again: ~60 candidates per particle instead
// of ~300. Because the list keeps the walk order and drops only pairs that contribute exactly zero, the
// sums are the reference's sums in the reference's order.
//
// Exactness conditions, checked on the device:
//   - sweeps at the current positions x (normal, force, pressure force) need |x_i - x_j| <= h, always in
//     the list;
//   - the pressure sweep measures distances between predicted positions x*. A pair with
//     |x*_i - x*_j| <= h has |x_i - x_j| <= h + |x*_i - x_i| + |x*_j - x_j|, so it is in both lists when
//     both displacements are at most half the skin. A particle whose displacement exceeds that ("fast")
//     flags its own bucket when it predicts x*. In a pressure sweep after any fast prediction, a particle
//     whose 27 buckets include a flagged one walks the buckets instead of using its list: every pair with a
//     fast particle j in i's walk (spatial neighbour or hash collision) is then summed by a walk. Flags
//     last for the rest of the step;
//   - a particle with more than list_cap candidates is marked (count > cap) and walks the buckets.
// Boundary particles (B > 0) are summed by walking the boundary buckets, as in the other variants.
//
// All arrays stay in the reference's sorted order (hash order, which scatters neighbouring cells across
// memory). Threads are mapped to particles through a "working order" instead: a permutation sorted by the
// Morton code of each particle's cell, so that the 32 particles of a warp are spatial neighbours and their
// neighbour gathers hit the same cache lines. Any permutation gives the same results (each particle's
// sum is independent of which thread computes it); the working order is only refreshed every few steps.
#include "pair_terms.cuh"
#include "step_kernels.cuh"

namespace pcisph {
namespace {

constexpr int kBlock = 256;
inline unsigned grid_for(uint32_t n) { return (n + kBlock - 1) / kBlock; }

// Particle handled by this thread (nullptr work: identity).
__device__ __forceinline__ uint32_t particle_of(const uint32_t* __restrict__ work, uint32_t t) {
    return work ? __ldg(&work[t]) : t;
}

// Spread the low 10 bits of v to every third bit (Morton interleave).
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 1023u;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Morton code of each particle's cell (low 10 bits per axis; locality only) and the identity values.
__global__ void __launch_bounds__(kBlock) k_morton(const float4* __restrict__ pos, uint32_t n, DevParams P,
                                                   uint32_t* __restrict__ code) {
    const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
    if (t >= n) return;
    const float4 x = pos[t];
    const Cell c = cell_of(x.x, x.y, x.z, P);
    code[t] = spread3(c.x) | (spread3(c.y) << 1) | (spread3(c.z) << 2);
}

// Call f(j) for every listed neighbour, four indices per 16-byte load (independent gathers in flight).
template <class F>
__device__ __forceinline__ void for_each_listed(const uint32_t* __restrict__ row, uint32_t n, F&& f) {
    const uint4* r4 = reinterpret_cast<const uint4*>(row);
    uint32_t k = 0;
#pragma unroll 1
    for (; k + 8 <= n; k += 8) {
        const uint4 q = __ldg(&r4[k >> 2]);
        const uint4 w = __ldg(&r4[(k >> 2) + 1]);
        f(q.x);
        f(q.y);
        f(q.z);
        f(q.w);
        f(w.x);
        f(w.y);
        f(w.z);
        f(w.w);
    }
    for (; k < n; ++k) f(__ldg(&row[k]));
}

// After predicting x*_i (stored as xs): record the step's max displacement; a fast particle flags its bucket.
__device__ __forceinline__ void note_displacement(const DevParams& P, Control* ctl,
                                                  unsigned char* __restrict__ bucket_fast, const float4& xi,
                                                  const float4& xs) {
    const float dx = xs.x - xi.x, dy = xs.y - xi.y, dz = xs.z - xi.z;  // exact: xs and xi are close
    const float disp = sqrtf(dx * dx + dy * dy + dz * dz);
    const unsigned act = __activemask();
    const unsigned m = __reduce_max_sync(act, __float_as_uint(disp));
    if ((int)(threadIdx.x & 31) == __ffs(act) - 1) atomicMax(&ctl->max_disp_bits, m);
    if (disp > P.list_half_skin) {
        atomicAdd(&ctl->fast_particles, 1ull);
        const Cell c = cell_of(xi.x, xi.y, xi.z, P);
        bucket_fast[hash_key(c.x, c.y, c.z, P)] = 1;
    }
}

// Does any of the 27 buckets around c hold a fast particle this step?
__device__ __forceinline__ bool near_fast(const DevParams& P, const unsigned char* __restrict__ bucket_fast, const Cell& c) {
    bool any = false;
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
                any |= bucket_fast[mod_bk(v & 0x7FFFFFFFu, P)] != 0;
            }
        }
    }
    return any;
}

// pcisph.cl:65-92, and the neighbour list of the step
__global__ void __launch_bounds__(kBlock) k_density_list(DevParams P, const uint2* __restrict__ b_cells,
                                                         const float4* __restrict__ b_pos,
                                                         const uint2* __restrict__ cells,
                                                         const float4* __restrict__ pos, float* __restrict__ rho,
                                                         float4* __restrict__ pr4, uint32_t* __restrict__ nbr,
                                                         uint32_t* __restrict__ nbr_count,
                                                         const uint32_t* __restrict__ work) {
    const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
    if (t >= P.fluid_count) return;
    const uint32_t i = particle_of(work, t);
    const float4 xi = pos[i];
    const Cell c = cell_of(xi.x, xi.y, xi.z, P);
    float acc = 0.f;
    if (P.boundary_count)
        for_each_neighbour(b_cells, c, P, [&](uint32_t j) { acc += density_term(xi.x, xi.y, xi.z, __ldg(&b_pos[j]), P.h2); });
    uint32_t* row = nbr + (size_t)i * P.list_cap;
    uint32_t n = 0;
    for_each_neighbour(cells, c, P, [&](uint32_t j) {
        const float4 o = __ldg(&pos[j]);
        const float dx = xi.x - o.x, dy = xi.y - o.y, dz = xi.z - o.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        acc += poly6(r2, P.h2);
        if (r2 <= P.list_r2) {
            if (n < P.list_cap) row[n] = j;
            ++n;
        }
    });
    nbr_count[i] = n;  // n > list_cap: this particle walks the buckets in the later sweeps
    acc *= P.particle_mass * P.poly6_norm;
    rho[i] = acc;
    pr4[i] = make_float4(xi.x, xi.y, xi.z, acc);
}

// pcisph.cl:94-112
__global__ void __launch_bounds__(kBlock) k_normal_list(DevParams P, const uint2* __restrict__ cells,
                                                        const float4* __restrict__ pr4, float4* __restrict__ normal,
                                                        const uint32_t* __restrict__ nbr,
                                                        const uint32_t* __restrict__ nbr_count,
                                                        const uint32_t* __restrict__ work) {
    const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
    if (t >= P.fluid_count) return;
    const uint32_t i = particle_of(work, t);
    const float4 xi = pr4[i];
    float3 n = make_float3(0.f, 0.f, 0.f);
    const uint32_t cnt = nbr_count[i];
    auto f = [&](uint32_t j) { normal_term(xi.x, xi.y, xi.z, __ldg(&pr4[j]), P.h2, n); };
    if (cnt <= P.list_cap) for_each_listed(nbr + (size_t)i * P.list_cap, cnt, f);
    else for_each_neighbour(cells, cell_of(xi.x, xi.y, xi.z, P), P, f);
    const float scale = P.h * P.particle_mass * P.poly6_d1_norm;
    normal[i] = make_float4(n.x * scale, n.y * scale, n.z * scale, 0.f);
}

// pcisph.cl:121-173, then the first predict (pcisph.cl:175-193, F_p = 0)
__global__ void __launch_bounds__(kBlock) k_force_list(DevParams P, const uint2* __restrict__ cells,
                                                       const float4* __restrict__ pr4, const float4* __restrict__ vel,
                                                       const float4* __restrict__ normal,
                                                       float4* __restrict__ f_other, float* __restrict__ press,
                                                       float4* __restrict__ pred, const uint32_t* __restrict__ nbr,
                                                       const uint32_t* __restrict__ nbr_count, Control* ctl,
                                                       const uint32_t* __restrict__ work,
                                                       unsigned char* __restrict__ bucket_fast) {
    const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
    if (t >= P.fluid_count) return;
    const uint32_t i = particle_of(work, t);
    const float4 xi = pr4[i];
    const float3 vi = f3(vel[i]);
    const float3 ni = f3(normal[i]);
    ForceAccum fa{make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f)};
    const uint32_t cnt = nbr_count[i];
    auto f = [&](uint32_t j) { force_term(xi, vi, ni, __ldg(&pr4[j]), f3(__ldg(&vel[j])), f3(__ldg(&normal[j])), P, fa); };
    if (cnt <= P.list_cap) for_each_listed(nbr + (size_t)i * P.list_cap, cnt, f);
    else for_each_neighbour(cells, cell_of(xi.x, xi.y, xi.z, P), P, f);
    const float m = P.particle_mass;
    const float3 visc = fa.visc * (P.viscosity * m * P.visc_d2_norm);
    const float3 coh = fa.coh * (-P.st_coeff * m * m * P.st_norm);
    const float3 curv = fa.curv * (-P.st_coeff * m);
    const float3 fo = make_float3(0.f, m * P.gravity, 0.f) + visc + (coh + curv);
    f_other[i] = f4(fo, 0.f);
    press[i] = 0.f;
    const float3 v = vi + (fo / m) * P.dt;
    const float3 dx = v * P.dt;
    const float4 xs = make_float4(xi.x + dx.x, xi.y + dx.y, xi.z + dx.z, 0.f);
    pred[i] = xs;
    note_displacement(P, ctl, bucket_fast, xi, xs);
}

// pcisph.cl:212-263 (boundary_update = 0) + the stop decision (Fluid.cpp:284-306)
__global__ void __launch_bounds__(kBlock) k_pressure_list(DevParams P, const uint2* __restrict__ b_cells,
                                                          const float4* __restrict__ b_pos,
                                                          const uint2* __restrict__ cells,
                                                          const float4* __restrict__ pos,
                                                          const float4* __restrict__ pred,
                                                          const float* __restrict__ rho, float* __restrict__ press,
                                                          float* __restrict__ err, float4* __restrict__ pf4,
                                                          const uint32_t* __restrict__ nbr,
                                                          const uint32_t* __restrict__ nbr_count, Control* ctl,
                                                          const uint32_t* __restrict__ work,
                                                          const unsigned char* __restrict__ bucket_fast) {
    const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
    // no particle moved more than half the skin: every list is complete for x* (no marks were made)
    const bool all_lists_ok = __uint_as_float(*(volatile unsigned*)&ctl->max_disp_bits) <= P.list_half_skin;
    float dv = 0.f;
    if (t < P.fluid_count) {
        const uint32_t i = particle_of(work, t);
        const float4 xi = pos[i];
        const float4 xp = pred[i];
        float acc = 0.f;
        const uint32_t cnt = nbr_count[i];
        const Cell c = cell_of(xi.x, xi.y, xi.z, P);
        const bool walk = cnt > P.list_cap || (!all_lists_ok && near_fast(P, bucket_fast, c));
        if (P.boundary_count)
            for_each_neighbour(b_cells, c, P, [&](uint32_t j) { acc += density_term(xp.x, xp.y, xp.z, __ldg(&b_pos[j]), P.h2); });
        auto f = [&](uint32_t j) { acc += density_term(xp.x, xp.y, xp.z, __ldg(&pred[j]), P.h2); };
        if (walk) for_each_neighbour(cells, c, P, f);
        else for_each_listed(nbr + (size_t)i * P.list_cap, cnt, f);
        acc *= P.particle_mass * P.poly6_norm;
        if (!isfinite(acc)) atomicOr(&ctl->status, 2u);
        dv = acc - P.rest_density;
        dv = 0.f < dv ? dv : 0.f;
        err[i] = dv;
        float p = press[i];
        if (dv != 0.f) {
            p += dv * P.delta;
            press[i] = p;
        }
        const float r = rho[i];
        pf4[i] = make_float4(xi.x, xi.y, xi.z, p / (r * r));
    }
    unsigned bits = __reduce_max_sync(0xffffffffu, __float_as_uint(dv));
    __shared__ unsigned warp_max[kBlock / 32];
    __shared__ bool is_last;
    if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = bits;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned m = 0;
#pragma unroll
        for (int w = 0; w < kBlock / 32; ++w) m = max(m, warp_max[w]);
        atomicMax(&ctl->max_err_bits, m);
        __threadfence();
        is_last = atomicAdd(&ctl->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (is_last && threadIdx.x == 0) {
        __threadfence();
        const float mx = __uint_as_float(atomicAdd(&ctl->max_err_bits, 0u));
        const unsigned it = ctl->iter + 1;
        const float rel = mx / P.rest_density;
        const bool converged = rel < P.threshold;
        const bool done = it >= (unsigned)P.max_iters || (it >= (unsigned)P.min_iters && converged);
        ctl->iter = it;
        ctl->done = done ? 1u : 0u;
        ctl->max_err_bits = 0;
        ctl->blocks_done = 0;
        if (!all_lists_ok) ctl->list_fallbacks += 1;
        if (done) {
            if (!converged) ctl->status |= 1u;
            ctl->status_all |= ctl->status;
            ctl->iterations_last = (int)it;
            ctl->max_err_last = rel;
            ctl->steps += 1;
            ctl->total_iters += it;
        }
    }
}

// pcisph.cl:265-300, then predict (pcisph.cl:175-193) or integrate with optional walls
__global__ void __launch_bounds__(kBlock) k_pressure_force_list(
    DevParams P, const uint2* __restrict__ b_cells, const float4* __restrict__ bpf, const uint2* __restrict__ cells,
    const float4* __restrict__ pf4, const float4* __restrict__ vel, const float4* __restrict__ f_other,
    float4* __restrict__ f_press, float4* __restrict__ pred, float4* __restrict__ state_pos,
    float4* __restrict__ state_vel, const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ nbr_count,
    Control* ctl, int mode, cudaGraphConditionalHandle cond, int use_cond, const uint32_t* __restrict__ work,
    unsigned char* __restrict__ bucket_fast) {
    const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
    if (use_cond && t == 0) {
        // continue the graph's while loop unless the step is done; the counter bounds it on its own
        const unsigned g = ++ctl->guard_iters;
        const bool stop = ctl->done != 0u || g >= (unsigned)P.max_iters;
        cudaGraphSetConditional(cond, stop ? 0u : 1u);
    }
    if (t >= P.fluid_count) return;
    const uint32_t i = particle_of(work, t);
    const float4 xi = pf4[i];
    float3 f = make_float3(0.f, 0.f, 0.f);
    const uint32_t cnt = nbr_count[i];
    Cell c{0u, 0u, 0u};
    if (cnt > P.list_cap || P.boundary_count) c = cell_of(xi.x, xi.y, xi.z, P);
    if (P.boundary_count)
        for_each_neighbour(b_cells, c, P, [&](uint32_t j) { pressure_force_term(xi, __ldg(&bpf[j]), P.h, P.h2, f); });
    auto body = [&](uint32_t j) { pressure_force_term(xi, __ldg(&pf4[j]), P.h, P.h2, f); };
    if (cnt <= P.list_cap) for_each_listed(nbr + (size_t)i * P.list_cap, cnt, body);
    else for_each_neighbour(cells, c, P, body);
    const float m = P.particle_mass;
    const float scale = -P.spiky_d1_norm * m * m;
    const float3 fp = make_float3(f.x * scale, f.y * scale, f.z * scale);
    f_press[i] = f4(fp, 0.f);
    const bool integrate = mode == 0 ? (ctl->done != 0u) : mode == 2;
    const float3 a = (f3(f_other[i]) + fp) / m;
    float3 v = f3(vel[i]) + a * P.dt;
    const float3 dx = v * P.dt;
    float3 x = make_float3(xi.x + dx.x, xi.y + dx.y, xi.z + dx.z);
    if (!integrate) {
        const float4 xs = f4(x, 0.f);
        pred[i] = xs;
        note_displacement(P, ctl, bucket_fast, xi, xs);
        return;
    }
    if (P.walls) {
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            float* xs = ax == 0 ? &x.x : ax == 1 ? &x.y : &x.z;
            float* vs = ax == 0 ? &v.x : ax == 1 ? &v.y : &v.z;
            if (*xs < P.box_lo[ax]) {
                *xs = P.box_lo[ax];
                if (*vs < 0.f) *vs = -P.restitution * *vs;
            } else if (*xs > P.box_hi[ax]) {
                *xs = P.box_hi[ax];
                if (*vs > 0.f) *vs = -P.restitution * *vs;
            }
        }
    }
    state_pos[i] = f4(x, 0.f);
    state_vel[i] = f4(v, 0.f);
}

}  // namespace

__global__ void __launch_bounds__(kBlock) k_iota(uint32_t* __restrict__ out, uint32_t n) {
    const uint32_t t = blockIdx.x * kBlock + threadIdx.x;
    if (t < n) out[t] = t;
}

void launch_iota(uint32_t* out, uint32_t n, cudaStream_t s) {
    if (n) k_iota<<<grid_for(n), kBlock, 0, s>>>(out, n);
}

void launch_morton(const float4* pos, uint32_t n, const DevParams& P, uint32_t* code, cudaStream_t s) {
    if (n) k_morton<<<grid_for(n), kBlock, 0, s>>>(pos, n, P, code);
}

void launch_density_list(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    k_density_list<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.b_cells, b.b_pos, b.cells, b.pos, b.rho, b.pr4, b.nbr,
                                                               b.nbr_count, b.work);
}
void launch_normal_list(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    k_normal_list<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.cells, b.pr4, b.normal, b.nbr, b.nbr_count, b.work);
}
void launch_force_list(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    k_force_list<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.cells, b.pr4, b.vel, b.normal, b.f_other, b.press, b.pred,
                                                             b.nbr, b.nbr_count, b.ctl, b.work, b.bucket_fast);
}
void launch_pressure_list(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    k_pressure_list<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.b_cells, b.b_pos, b.cells, b.pos, b.pred, b.rho,
                                                                b.press, b.err, b.pf4, b.nbr, b.nbr_count, b.ctl, b.work,
                                                                b.bucket_fast);
}
void launch_pressure_force_list(const DevParams& P, const StepBuffers& b, int mode, cudaGraphConditionalHandle cond,
                                bool use_cond, cudaStream_t s) {
    k_pressure_force_list<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.b_cells, b.bpf, b.cells, b.pf4, b.vel,
                                                                      b.f_other, b.f_press, b.pred, b.state_pos,
                                                                      b.state_vel, b.nbr, b.nbr_count, b.ctl, mode,
                                                                      cond, use_cond ? 1 : 0, b.work, b.bucket_fast);
}

}  // namespace pcisph
