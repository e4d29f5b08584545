// step_kernels.cu -- the PCISPH step on sm_103a.
//
// One thread per particle walks the reference's 27 hashed buckets
// (PCISPH/data/kernels/grid_utils.cl:65-79) with coalesced float4 loads of
// packed neighbour operands. Every pair term is the reference's expression
// (PCISPH/data/kernels/pcisph.cl); pairs farther than h contribute exactly zero
// in every reference kernel, so the per-pair work is skipped for them.
//
// Fusions relative to the reference's kernel list (Fluid.cpp:212-316):
//   density        also writes pr4 = (x, rho)
//   force          also zeroes p and does the first predict (F_p = 0 there)
//   pressure       also writes pf4 = (x, p/rho^2), reduces the max density
//                  variation and, in the last block, decides whether the loop
//                  stops (the reference reads err[] back and decides on the host)
//   pressure force then predicts for the next iteration, or integrates (with
//                  optional walls) when the loop has stopped
#include "step_kernels.cuh"
#include "pair_terms.cuh"
#include "sweep.cuh"

namespace pcisph {
namespace {

constexpr int kBlock = 256;

inline unsigned grid_for(uint32_t n) { return (n + kBlock - 1) / kBlock; }

template <bool PACKED>
__global__ void __launch_bounds__(kBlock) k_hash(const float* __restrict__ pos, uint32_t n, DevParams P,
                                                 uint32_t* __restrict__ keys, uint32_t* __restrict__ ids) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    float x, y, z;
    if (PACKED) {
        x = pos[3 * (size_t)i];
        y = pos[3 * (size_t)i + 1];
        z = pos[3 * (size_t)i + 2];
    } else {
        const float4 p = reinterpret_cast<const float4*>(pos)[i];
        x = p.x; y = p.y; z = p.z;
    }
    const Cell c = cell_of(x, y, z, P);
    keys[i] = P.bucket_base + hash_key(c.x, c.y, c.z, P);
    if (ids) ids[i] = i;
}

// sort_utils.cl:51-78 (cells were cleared before, sort_utils.cl:7-10). Also the cell code of each
// particle and the list of bucket-run starts that the warp sweeps iterate.
__global__ void __launch_bounds__(kBlock) k_reorder(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ ids,
                                                    const float4* __restrict__ in_pos,
                                                    const float4* __restrict__ in_vel, uint32_t n,
                                                    float4* __restrict__ out_pos, float4* __restrict__ out_vel,
                                                    uint2* __restrict__ cells, uint32_t* __restrict__ codes,
                                                    uint32_t* __restrict__ groups, DevParams P, Control* ctl,
                                                    const float* __restrict__ in_skin) {
    const uint32_t d = blockIdx.x * kBlock + threadIdx.x;
    if (d >= n) return;
    const uint32_t src = ids[d];
    const uint32_t key = keys[d];
    const bool ok = src < n && key < P.bucket_count;
    bool is_start = false;
    if (ok) {
        float4 p = in_pos[src];
        if (in_skin) p.w = in_skin[src];  // the particle's stored half skin rides in w
        out_pos[d] = p;
        if (in_vel) out_vel[d] = in_vel[src];
        if (codes) {
            const Cell c = cell_of(p.x, p.y, p.z, P);
            codes[d] = cell_code(c.x, c.y, c.z);
        }
        is_start = d == 0 || key != keys[d - 1];
        if (is_start) cells[key].x = d;
        if (d == n - 1 || key != keys[d + 1]) cells[key].y = d + 1;
    } else if (ctl) {  // a sort that broke its contract: flag it, touch nothing
        atomicOr(&ctl->status, 4u);
    }
    if (groups) {
        const unsigned act = __activemask();
        const unsigned m = __ballot_sync(act, is_start);
        if (m) {
            const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&ctl->n_groups, (unsigned)__popc(m));
            base = __shfl_sync(act, base, leader);
            if (is_start) groups[base + __popc(m & ((1u << lane) - 1u))] = d;
        }
    }
}

__global__ void k_begin(Control* ctl) {
    ctl->iter = 0;
    ctl->done = 0;
    ctl->max_err_bits = 0;
    ctl->blocks_done = 0;
    ctl->status = 0;
    ctl->guard_iters = 0;
    ctl->n_groups = 0;
    ctl->fast_at_begin = ctl->fast_particles;
    ctl->fast_n = 0;
}

// pcisph.cl:65-92
__global__ void __launch_bounds__(kBlock) k_density(DevParams P, const uint2* __restrict__ b_cells,
                                                    const float4* __restrict__ b_pos, const uint2* __restrict__ cells,
                                                    const float4* __restrict__ pos, float* __restrict__ rho,
                                                    float4* __restrict__ pr4) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= P.fluid_count) return;
    const float4 xi = pos[i];
    const Cell c = cell_of(xi.x, xi.y, xi.z, P);
    const float h2 = P.h2;
    float acc = 0.f;
    if (P.boundary_count) {
        for_each_neighbour(b_cells, c, P, [&](uint32_t j) {
            const float4 o = __ldg(&b_pos[j]);
            const float dx = xi.x - o.x, dy = xi.y - o.y, dz = xi.z - o.z;
            acc += poly6(dist2(dx, dy, dz), h2);
        });
    }
    for_each_neighbour(cells, c, P, [&](uint32_t j) {
        const float4 o = __ldg(&pos[j]);
        const float dx = xi.x - o.x, dy = xi.y - o.y, dz = xi.z - o.z;
        acc += poly6(dist2(dx, dy, dz), h2);
    });
    acc *= P.particle_mass * P.poly6_norm;
    rho[i] = acc;
    pr4[i] = make_float4(xi.x, xi.y, xi.z, acc);
}

// pcisph.cl:94-112
__global__ void __launch_bounds__(kBlock) k_normal(DevParams P, const uint2* __restrict__ cells,
                                                   const float4* __restrict__ pr4, float4* __restrict__ normal) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= P.fluid_count) return;
    const float4 xi = pr4[i];
    const Cell c = cell_of(xi.x, xi.y, xi.z, P);
    const float h2 = P.h2;
    float3 n = make_float3(0.f, 0.f, 0.f);
    for_each_neighbour(cells, c, P, [&](uint32_t j) { normal_term(xi.x, xi.y, xi.z, __ldg(&pr4[j]), h2, n); });
    const float scale = P.h * P.particle_mass * P.poly6_d1_norm;
    normal[i] = make_float4(n.x * scale, n.y * scale, n.z * scale, 0.f);
}

// pcisph.cl:121-173, then pcisph.cl:175-193 with F_p = 0 (the first predict)
__global__ void __launch_bounds__(kBlock) k_force(DevParams P, const uint2* __restrict__ cells,
                                                  const float4* __restrict__ pr4, const float4* __restrict__ vel,
                                                  const float4* __restrict__ normal, float4* __restrict__ f_other,
                                                  float* __restrict__ press, float4* __restrict__ pred) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= P.fluid_count) return;
    const float4 xi = pr4[i];
    const float3 vi = f3(vel[i]);
    const float3 ni = f3(normal[i]);
    const Cell c = cell_of(xi.x, xi.y, xi.z, P);
    ForceAccum fa{make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f)};
    for_each_neighbour(cells, c, P, [&](uint32_t j) {
        force_term(xi, vi, ni, __ldg(&pr4[j]), f3(__ldg(&vel[j])), f3(__ldg(&normal[j])), P, fa);
    });
    const float m = P.particle_mass;
    const float3 fo = other_force(m, P.gravity, fa.visc, P.viscosity * m * P.visc_d2_norm, fa.coh,
                                  -P.st_coeff * m * m * P.st_norm, fa.curv, -P.st_coeff * m);
    f_other[i] = f4(fo, 0.f);
    press[i] = 0.f;
    const float3 a = fo / m;
    const float3 v = vi + a * P.dt;
    const float3 x = make_float3(xi.x, xi.y, xi.z) + v * P.dt;
    pred[i] = f4(x, 0.f);
}

// pcisph.cl:195-210 (raw sum, no m*K factor)
__global__ void __launch_bounds__(kBlock) k_boundary_self_density(DevParams P, const uint2* __restrict__ b_cells,
                                                                  const float4* __restrict__ b_pos,
                                                                  float* __restrict__ b_init) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= P.boundary_count) return;
    const float4 xi = b_pos[i];
    const Cell c = cell_of(xi.x, xi.y, xi.z, P);
    float acc = 0.f;
    for_each_neighbour(b_cells, c, P, [&](uint32_t j) {
        const float4 o = __ldg(&b_pos[j]);
        const float dx = xi.x - o.x, dy = xi.y - o.y, dz = xi.z - o.z;
        acc += poly6(dist2(dx, dy, dz), P.h2);
    });
    b_init[i] = acc;
}

// pcisph.cl:212-263 with boundary_update = 1
__global__ void __launch_bounds__(kBlock) k_boundary_pressure(DevParams P, const uint2* __restrict__ cells,
                                                              const float4* __restrict__ pred,
                                                              const float4* __restrict__ b_pos,
                                                              const float* __restrict__ b_init,
                                                              float* __restrict__ b_press,
                                                              float4* __restrict__ bpf) {
    boundary_pressure_body(P, cells, pred, b_pos, b_init, b_press, bpf, blockIdx.x * kBlock + threadIdx.x);
}

// pcisph.cl:212-263 with boundary_update = 0, plus the stop decision (Fluid.cpp:284-306)
__global__ void __launch_bounds__(kBlock) k_pressure(DevParams P, const uint2* __restrict__ b_cells,
                                                     const float4* __restrict__ b_pos, const uint2* __restrict__ cells,
                                                     const float4* __restrict__ pos, const float4* __restrict__ pred,
                                                     const float* __restrict__ rho, float* __restrict__ press,
                                                     float* __restrict__ err, float4* __restrict__ pf4, Control* ctl) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    float dv = 0.f;
    if (i < P.fluid_count) {
        const float4 xi = pos[i];
        const float4 xp = pred[i];
        const Cell c = cell_of(xi.x, xi.y, xi.z, P);
        const float h2 = P.h2;
        float acc = 0.f;
        if (P.boundary_count) {
            for_each_neighbour(b_cells, c, P, [&](uint32_t j) {
                const float4 o = __ldg(&b_pos[j]);
                const float dx = xp.x - o.x, dy = xp.y - o.y, dz = xp.z - o.z;
                acc += poly6(dist2(dx, dy, dz), h2);
            });
        }
        for_each_neighbour(cells, c, P, [&](uint32_t j) {
            const float4 o = __ldg(&pred[j]);
            const float dx = xp.x - o.x, dy = xp.y - o.y, dz = xp.z - o.z;
            acc += poly6(dist2(dx, dy, dz), h2);
        });
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
    // block max of dv (dv >= 0, so its bit pattern orders like the value)
    unsigned bits = __float_as_uint(dv);
    bits = __reduce_max_sync(0xffffffffu, bits);
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
        if (done) close_step(ctl, it, rel, converged);
    }
}

// pcisph.cl:265-300, then pcisph.cl:175-193: predict x* or integrate x, v (+ walls)
__global__ void __launch_bounds__(kBlock) k_pressure_force(DevParams P, const uint2* __restrict__ b_cells,
                                                           const float4* __restrict__ bpf,
                                                           const uint2* __restrict__ cells,
                                                           const float4* __restrict__ pf4,
                                                           const float4* __restrict__ vel,
                                                           const float4* __restrict__ f_other,
                                                           float4* __restrict__ f_press, float4* __restrict__ pred,
                                                           float4* __restrict__ state_pos,
                                                           float4* __restrict__ state_vel, Control* ctl, int mode,
                                                           cudaGraphConditionalHandle cond, int use_cond) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (use_cond && i == 0) {
        // The graph's while loop continues only if this returns 1. The decision of the pressure kernel is
        // final here (that kernel has completed); the separate counter bounds the loop at max_iters on
        // its own, so the loop ends even if the decision were never written.
        const unsigned g = ++ctl->guard_iters;
        const bool stop = ctl->done != 0u || g >= (unsigned)P.max_iters;
        cudaGraphSetConditional(cond, stop ? 0u : 1u);
    }
    if (i >= P.fluid_count) return;
    const float4 xi = pf4[i];
    const Cell c = cell_of(xi.x, xi.y, xi.z, P);
    float3 f = make_float3(0.f, 0.f, 0.f);
    if (P.boundary_count)
        for_each_neighbour(b_cells, c, P, [&](uint32_t j) { pressure_force_term(xi, __ldg(&bpf[j]), P.h, P.h2, f); });
    for_each_neighbour(cells, c, P, [&](uint32_t j) { pressure_force_term(xi, __ldg(&pf4[j]), P.h, P.h2, f); });
    const float m = P.particle_mass;
    const float scale = -P.spiky_d1_norm * m * m;
    const float3 fp = make_float3(f.x * scale, f.y * scale, f.z * scale);
    f_press[i] = f4(fp, 0.f);
    const bool integrate = mode == 0 ? (ctl->done != 0u) : mode == 2;
    const float3 fo = f3(f_other[i]);
    const float3 a = (fo + fp) / m;
    float3 v = f3(vel[i]) + a * P.dt;
    float3 x = make_float3(xi.x, xi.y, xi.z) + v * P.dt;
    if (!integrate) {
        pred[i] = f4(x, 0.f);
        return;
    }
    if (P.walls) {
        float* xs[3] = {&x.x, &x.y, &x.z};
        float* vs[3] = {&v.x, &v.y, &v.z};
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
            if (*xs[ax] < P.box_lo[ax]) {
                *xs[ax] = P.box_lo[ax];
                if (*vs[ax] < 0.f) *vs[ax] = -P.restitution * *vs[ax];
            } else if (*xs[ax] > P.box_hi[ax]) {
                *xs[ax] = P.box_hi[ax];
                if (*vs[ax] > 0.f) *vs[ax] = -P.restitution * *vs[ax];
            }
        }
    }
    state_pos[i] = f4(x, 0.f);
    state_vel[i] = f4(v, 0.f);
}

// Rebuild pr4 from (pos, rho) and pf4 from (pos, press, rho) after fields were overwritten.
__global__ void __launch_bounds__(kBlock) k_pack(DevParams P, const float4* __restrict__ pos,
                                                 const float* __restrict__ rho, const float* __restrict__ press,
                                                 float4* __restrict__ pr4, float4* __restrict__ pf4) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= P.fluid_count) return;
    const float4 x = pos[i];
    const float r = rho[i];
    pr4[i] = make_float4(x.x, x.y, x.z, r);
    pf4[i] = make_float4(x.x, x.y, x.z, press[i] / (r * r));
}

__global__ void __launch_bounds__(kBlock) k_pack_boundary(DevParams P, const float4* __restrict__ b_pos,
                                                          const float* __restrict__ b_press,
                                                          float4* __restrict__ bpf) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= P.boundary_count) return;
    const float4 x = b_pos[i];
    bpf[i] = make_float4(x.x, x.y, x.z, b_press[i] / (P.rest_density * P.rest_density));
}

// Packed float3 <-> float4. A block moves its 256 elements' 768 packed floats as three fully coalesced
// rows (thread t: floats t, t + 256, t + 512) through shared memory (stride-3 element access there is
// conflict-free), so every request covers whole 128-byte lines: this matters most when the packed side is
// pinned host memory read or written over the host link.
__global__ void __launch_bounds__(kBlock) k_pack3_to4(const float* __restrict__ in3, float4* __restrict__ out,
                                                      uint32_t n) {
    __shared__ float tile[3 * kBlock];
    const size_t base = (size_t)blockIdx.x * kBlock;
    const size_t total = 3 * (size_t)n;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const size_t k = 3 * base + r * kBlock + threadIdx.x;
        if (k < total) tile[r * kBlock + threadIdx.x] = in3[k];
    }
    __syncthreads();
    const size_t i = base + threadIdx.x;
    if (i < n) {
        const float* e = &tile[3 * threadIdx.x];
        out[i] = make_float4(e[0], e[1], e[2], 0.f);
    }
}

__global__ void __launch_bounds__(kBlock) k_unpack4_to3(const float4* __restrict__ in, float* __restrict__ out3,
                                                        uint32_t n) {
    __shared__ float tile[3 * kBlock];
    const size_t base = (size_t)blockIdx.x * kBlock;
    const size_t i = base + threadIdx.x;
    if (i < n) {
        const float4 v = in[i];
        float* e = &tile[3 * threadIdx.x];
        e[0] = v.x;
        e[1] = v.y;
        e[2] = v.z;
    }
    __syncthreads();
    const size_t total = 3 * (size_t)n;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const size_t k = 3 * base + r * kBlock + threadIdx.x;
        if (k < total) out3[k] = tile[r * kBlock + threadIdx.x];
    }
}

}  // namespace

void launch_hash(const float* pos, bool packed, uint32_t n, const DevParams& P, uint32_t* keys, uint32_t* ids,
                 cudaStream_t s) {
    if (!n) return;
    if (packed) k_hash<true><<<grid_for(n), kBlock, 0, s>>>(pos, n, P, keys, ids);
    else k_hash<false><<<grid_for(n), kBlock, 0, s>>>(pos, n, P, keys, ids);
}

void launch_reorder(const uint32_t* keys, const uint32_t* ids, const float4* in_pos, const float4* in_vel,
                    uint32_t n, float4* out_pos, float4* out_vel, uint2* cells, uint32_t* codes, uint32_t* groups,
                    const DevParams& P, Control* ctl, cudaStream_t s, const float* in_skin) {
    if (!n) return;
    k_reorder<<<grid_for(n), kBlock, 0, s>>>(keys, ids, in_pos, in_vel, n, out_pos, out_vel, cells, codes, groups, P,
                                             ctl, in_skin);
}

void launch_begin(Control* ctl, cudaStream_t s) { k_begin<<<1, 1, 0, s>>>(ctl); }

void launch_density(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    k_density<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.b_cells, b.b_pos, b.cells, b.pos, b.rho, b.pr4);
}

void launch_normal(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    k_normal<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.cells, b.pr4, b.normal);
}

void launch_force(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    k_force<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.cells, b.pr4, b.vel, b.normal, b.f_other, b.press,
                                                         b.pred);
}

void launch_boundary_self_density(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    if (!P.boundary_count) return;
    k_boundary_self_density<<<grid_for(P.boundary_count), kBlock, 0, s>>>(P, b.b_cells, b.b_pos, b.b_init);
}

void launch_boundary_pressure(const DevParams& P, const StepBuffers& b, const uint2* cells, cudaStream_t s) {
    if (!P.boundary_count) return;
    k_boundary_pressure<<<grid_for(P.boundary_count), kBlock, 0, s>>>(P, cells, b.pred, b.b_pos, b.b_init,
                                                                       b.b_press, b.bpf);
}

void launch_pressure(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    k_pressure<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.b_cells, b.b_pos, b.cells, b.pos, b.pred, b.rho,
                                                            b.press, b.err, b.pf4, b.ctl);
}

void launch_pressure_force(const DevParams& P, const StepBuffers& b, int mode, cudaGraphConditionalHandle cond,
                           bool use_cond, cudaStream_t s) {
    k_pressure_force<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.b_cells, b.bpf, b.cells, b.pf4, b.vel,
                                                                  b.f_other, b.f_press, b.pred, b.state_pos,
                                                                  b.state_vel, b.ctl, mode, cond, use_cond ? 1 : 0);
}

void launch_pack(const DevParams& P, const StepBuffers& b, cudaStream_t s) {
    k_pack<<<grid_for(P.fluid_count), kBlock, 0, s>>>(P, b.pos, b.rho, b.press, b.pr4, b.pf4);
    if (P.boundary_count)
        k_pack_boundary<<<grid_for(P.boundary_count), kBlock, 0, s>>>(P, b.b_pos, b.b_press, b.bpf);
}

void launch_pack3_to4(const float* in3, float4* out, uint32_t n, cudaStream_t s) {
    if (n) k_pack3_to4<<<grid_for(n), kBlock, 0, s>>>(in3, out, n);
}

void launch_unpack4_to3(const float4* in, float* out3, uint32_t n, cudaStream_t s) {
    if (n) k_unpack4_to3<<<grid_for(n), kBlock, 0, s>>>(in, out3, n);
}

}  // namespace pcisph
