// pair_terms.cuh -- the per-pair terms of the neighbour sweeps (PCISPH/data/kernels/pcisph.cl:8-300).
//
// Every term keeps the reference's expression and cut-offs. Two changes of arithmetic only:
//   - 1/r and r come from the approximate reciprocal square root (rsqrtf, <= 2 ulp) instead of an IEEE
//     sqrtf and division, and divisions by densities use __fdividef (<= 2 ulp). The reference itself uses
//     fast_length, which OpenCL allows to be approximate. Errors stay near 1e-7 relative per term, far
//     inside the 1e-5 parity bound; the cost per in-range pair drops from ~50 to ~10 instructions.
//   - pairs with r^2 > h^2 are skipped: every reference kernel returns exactly 0 for them (the force term
//     also looks at pairs within a few ulp beyond h, for its curvature cut-off: see force_term).
#pragma once
#include "common.cuh"

namespace pcisph {

// poly6 for density and predicted density (pcisph.cl:8-16, :80, :242, :250)
__device__ __forceinline__ float density_term(float xi, float yi, float zi, const float4& o, float h2) {
    const float dx = xi - o.x, dy = yi - o.y, dz = zi - o.z;
    return poly6(dist2(dx, dy, dz), h2);
}

// poly6 gradient over the neighbour's density (pcisph.cl:18-26, :107); o = (x_j, rho_j)
__device__ __forceinline__ void normal_term(float xi, float yi, float zi, const float4& o, float h2, float3& n) {
    const float dx = xi - o.x, dy = yi - o.y, dz = zi - o.z;
    const float r2 = dist2(dx, dy, dz);
    if (r2 <= h2) {
        const float k = __fdividef((r2 - h2) * (r2 - h2), o.w);
        n.x += dx * k;
        n.y += dy * k;
        n.z += dz * k;
    }
}

// viscosity and Akinci cohesion + curvature (pcisph.cl:137-159); xi = (x_i, rho_i), o = (x_j, rho_j)
struct ForceAccum {
    float3 visc, coh, curv;
};
__device__ __forceinline__ void force_term(const float4& xi, const float3& vi, const float3& ni, const float4& o,
                                           const float3& vj, const float3& nj, const DevParams& P,
                                           ForceAccum& a) {
    const float dx = xi.x - o.x, dy = xi.y - o.y, dz = xi.z - o.z;
    const float r2 = dist2(dx, dy, dz);
    // The curvature term does not vanish at r = h: it jumps to zero there. Within a few ulp of the cut-off the
    // decision is taken on the length as the oracle forms it (dot product rounded term by term, correctly
    // rounded sqrtf: its reading of the reference's fast_length), so that both land on the same side of h; a
    // lattice at spacing h/2, like the reference's voxel scenes, has many pairs at r = h.
    const bool at_cut = fabsf(r2 - P.h2) <= 1e-6f * P.h2;
    if (r2 <= P.h2 || at_cut) {
        const float inv_r = r2 > 0.f ? rsqrtf(r2) : 0.f;
        const float dist = __fmul_rn(r2, inv_r);  // rounded once: it has several uses
        const float rj = o.w;
        if (r2 <= P.h2 && rj > 0.0001f) {
            const float k = __fdividef(__fsub_rn(P.h, dist), rj);  // kernel_viscosity_d2 / rho_j
            a.visc.x += (vj.x - vi.x) * k;
            a.visc.y += (vj.y - vi.y) * k;
            a.visc.z += (vj.z - vi.z) * k;
        }
        const float d_cut =
            at_cut ? __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz))) : dist;
        if (dist > 0.0001f && d_cut < P.h) {
            const float corr = __fdividef(2.f * P.rest_density, xi.w + rj);
            const float c = corr * surface_tension_kernel(dist, P.h, P.st_term) * inv_r;  // * (x_i - x_j)/r
            a.coh.x += c * dx;
            a.coh.y += c * dy;
            a.coh.z += c * dz;
            a.curv.x += corr * (ni.x - nj.x);
            a.curv.y += corr * (ni.y - nj.y);
            a.curv.z += corr * (ni.z - nj.z);
        }
    }
}

// spiky gradient times (p_i/rho_i^2 + p_j/rho_j^2) (pcisph.cl:28-37, :279-295); xi.w, o.w = p/rho^2
__device__ __forceinline__ void pressure_force_term(const float4& xi, const float4& o, float h, float h2, float3& f) {
    const float dx = xi.x - o.x, dy = xi.y - o.y, dz = xi.z - o.z;
    const float r2 = dist2(dx, dy, dz);
    if (r2 <= h2 && r2 >= 1e-8f) {  // 1e-4 <= r <= h
        const float inv_r = rsqrtf(r2);
        const float dr = __fmaf_rn(-r2, inv_r, h);
        const float k = dr * dr * inv_r * (xi.w + o.w);
        f.x += dx * k;
        f.y += dy * k;
        f.z += dz * k;
    }
}

// One fluid particle's term in a boundary particle's predicted density (pcisph.cl:240-250 from the boundary
// side: distance from x_b to the fluid particle's predicted position)
__device__ __forceinline__ void boundary_density_term(const float4& xb, const float4& o, float h2, float& acc) {
    const float dx = xb.x - o.x, dy = xb.y - o.y, dz = xb.z - o.z;
    acc += poly6(dist2(dx, dy, dz), h2);
}

// The rest of a boundary particle's pressure update from its density sum acc (self density included):
// pressure increment delta * max(0, rho* - rho0) and the packed operand (x_b, p_b / rho0^2).
__device__ __forceinline__ void boundary_pressure_finish(const DevParams& P, const float4& xb, float acc,
                                                         float* __restrict__ b_press, float4* __restrict__ bpf,
                                                         uint32_t i) {
    acc *= P.particle_mass * P.poly6_norm;
    float dv = acc - P.rest_density;
    dv = 0.f < dv ? dv : 0.f;
    float p = b_press[i];
    if (dv != 0.f) {
        p += dv * P.delta;
        b_press[i] = p;
    }
    bpf[i] = make_float4(xb.x, xb.y, xb.z, p / (P.rest_density * P.rest_density));
}

// One boundary particle's pressure update at the predicted fluid positions (pcisph.cl:212-263 with
// boundary_update = 1): predicted density from its initial (self) density plus the fluid neighbours,
// pressure increment delta * max(0, rho* - rho0), and its packed operand (x_b, p_b / rho0^2) for the
// pressure force. cells: the fluid cell table in the order pred is stored in.
__device__ __forceinline__ void boundary_pressure_body(const DevParams& P, const uint2* __restrict__ cells,
                                                       const float4* __restrict__ pred,
                                                       const float4* __restrict__ b_pos,
                                                       const float* __restrict__ b_init, float* __restrict__ b_press,
                                                       float4* __restrict__ bpf, uint32_t i) {
    if (i >= P.boundary_count) return;
    const float4 xb = b_pos[i];
    const Cell c = cell_of(xb.x, xb.y, xb.z, P);
    float acc = b_init[i];
    for_each_neighbour(cells, c, P, [&](uint32_t j) { boundary_density_term(xb, __ldg(&pred[j]), P.h2, acc); });
    boundary_pressure_finish(P, xb, acc, b_press, bpf, i);
}

}  // namespace pcisph
