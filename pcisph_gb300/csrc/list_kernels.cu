// list_kernels.cu -- neighbour-list sweeps (kernel_variant 2), for one scene or a batch of scenes.
//
// The density sweep walks the reference's 27 buckets (grid_utils.cl:65-79) once per step and records,
// per particle and in walk order, two lists: every candidate j with |x_i - x_j| <= r_list = h (1 + skin),
// and the subset within h (plus a 1e-4 relative margin, far above rounding). The later sweeps of the step
// iterate a list instead of walking the buckets again: the sweeps at the current positions (normal,
// force, pressure force) the within-h list (~34 candidates), the pressure sweeps of the corrective
// iterations the skin list (~65-80), instead of the walk's ~210. Because a list keeps the walk order and
// drops only pairs that contribute exactly zero, the sums are the reference's sums in the reference's
// order.
//
// Exactness conditions, checked on the device:
//   - sweeps at the current positions x (normal, force, pressure force) need |x_i - x_j| <= h, always in
//     the within-h list;
//   - the pressure sweep measures distances between predicted positions x*. A pair with
//     |x*_i - x*_j| <= h has |x_i - x_j| <= h + |x*_i - x_i| + |x*_j - x_j|, so it is in both lists when
//     both displacements are at most half the skin. A particle whose displacement exceeds that ("fast")
//     flags its own bucket when it predicts x*. In a pressure sweep after any fast prediction, a particle
//     whose 27 buckets include a flagged one walks the buckets instead of using its list: every pair with a
//     fast particle j in i's walk (spatial neighbour or hash collision) is then summed by a walk. Flags
//     last for the rest of the step;
//   - a particle with more than list_cap (near_cap) candidates is marked (count > cap) and walks the
//     buckets in the sweeps that would use that list.
// Boundary particles (B > 0, single scene) are summed by walking the boundary buckets. The density sweep
// records per particle whether any boundary particle lies within r_list of x (b_near); boundary particles
// do not move, so a particle without one has only zero boundary terms in the pressure-force sweep (pairs
// within h of x) and, unless its prediction moved more than half the skin, in the pressure sweeps: those
// skip the boundary walk (27 bucket lookups and the hash-colliding boundary particles they hold).
//
// Parameter sources (list_kernels.cuh): OneScene passes one DevParams by value and the pressure kernel's
// last block decides the loop. SceneTable serves a batch: particle i belongs to scene scene_of[i], whose
// DevParams (own particle count, bucket count and base in the shared cell table, box, limits) and Control
// live in device tables. Scenes stay contiguous in the sorted arrays because each scene's keys occupy its
// own bucket range. k_batch_decide closes each iteration per scene; finished scenes skip the sweeps.
#include <cooperative_groups.h>

#include <algorithm>

#include "list_kernels.cuh"
#include "pair_terms.cuh"
#include "sweep_device.cuh"

namespace pcisph {
namespace {

constexpr int kBlock = 256;
inline unsigned grid_for(uint32_t n) { return (n + kBlock - 1) / kBlock; }
constexpr unsigned kMarkBlocks = 152;  // the marking kernel's grid (grid-stride over its items)

// List layout: entries k = 8c .. 8c+7 of particle i (chunk c) are 32 contiguous bytes at uint4 offset
// 2 (c * stride + i); chunks are column-major over particles. A warp's 32 consecutive particles read
// chunk c as 1 KB of contiguous memory, and the builder writes whole 32-byte sectors.
__device__ __forceinline__ uint4* list_chunk(uint32_t* list, uint32_t i, uint32_t c, uint32_t stride) {
    return reinterpret_cast<uint4*>(list) + 2 * ((size_t)c * stride + i);
}

// The builder stages each list's current chunk in shared memory, slot-major (buf[slot * kBlock + thread]:
// conflict-free whatever slot each lane is at), and writes whole chunks.
__device__ __forceinline__ void list_store_chunk(uint32_t* list, uint32_t i, uint32_t c, uint32_t stride,
                                                 const uint32_t* buf) {
    const uint32_t t = threadIdx.x;
    uint4* p = list_chunk(list, i, c, stride);
    __stcs(p, make_uint4(buf[t], buf[kBlock + t], buf[2 * kBlock + t], buf[3 * kBlock + t]));
    __stcs(p + 1, make_uint4(buf[4 * kBlock + t], buf[5 * kBlock + t], buf[6 * kBlock + t], buf[7 * kBlock + t]));
}

// Append j as entry k of particle i's list.
__device__ __forceinline__ void list_append(uint32_t* list, uint32_t i, uint32_t stride, uint32_t* buf, uint32_t k,
                                            uint32_t j) {
    buf[(k & 7u) * kBlock + threadIdx.x] = j;
    if ((k & 7u) == 7u) list_store_chunk(list, i, k >> 3, stride, buf);
}

// Write the last, partial chunk of a list of n <= cap entries.
__device__ __forceinline__ void list_finish(uint32_t* list, uint32_t i, uint32_t stride, const uint32_t* buf,
                                            uint32_t n, uint32_t cap) {
    if (n <= cap && (n & 7u)) list_store_chunk(list, i, n >> 3, stride, buf);
}

// One float4 of data that the step's kernels write: the read-only path, or (kCoherent) a plain load for data
// that other blocks of the same launch wrote before a grid barrier (the persistent loop), which the
// read-only path may serve stale.
template <bool kCoherent>
__device__ __forceinline__ float4 load_slot(const float4* p) {
    if constexpr (kCoherent) return *p;
    else return __ldg(p);
}

// Call f(j) for the n listed neighbours of particle i in list order. The next chunk's indices are loaded
// while the current chunk's eight gathers are in flight, so the list stream and the gathers overlap. The
// list loads are streaming (evict-first): the lists do not push the gathered particle data out of L2.
template <class F>
__device__ __forceinline__ void for_each_listed(const uint32_t* __restrict__ list, uint32_t i, uint32_t n,
                                                uint32_t stride, F&& f) {
    const uint32_t chunks = (n + 7u) >> 3;
    if (!chunks) return;
    const uint4* p = list_chunk(const_cast<uint32_t*>(list), i, 0, stride);
    const size_t step = 2 * (size_t)stride;
    uint4 a = __ldcs(p), b = __ldcs(p + 1);
#pragma unroll 1
    for (uint32_t c = 0; c < chunks; ++c) {
        uint4 na = make_uint4(0u, 0u, 0u, 0u), nb = na;
        if (c + 1 < chunks) {
            p += step;
            na = __ldcs(p);
            nb = __ldcs(p + 1);
        }
        const uint32_t left = n - 8u * c;  // entries in this chunk: min(8, left)
        const uint32_t e[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if ((uint32_t)u < left) f(e[u]);
        a = na;
        b = nb;
    }
}

// Does any of the 27 buckets around c hold a fast particle this step?
__device__ __forceinline__ bool near_fast(const DevParams& P, const unsigned char* __restrict__ bucket_fast,
                                          const Cell& c) {
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
                any |= bucket_fast[P.bucket_base + mod_bk(v & 0x7FFFFFFFu, P)] != 0;
            }
        }
    }
    return any;
}

// The fluid particles within r_list of boundary particle k at the step's start, in the order of the walk
// of pcisph.cl:212-263 with boundary_update = 1 (27 fluid buckets around the boundary particle's cell).
__global__ void __launch_bounds__(kBlock) k_boundary_fluid_list(DevParams P, ListBuffers b) {
    const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
    if (k >= P.boundary_count) return;
    const float4 xb = b.b_pos[k];
    const Cell c = cell_of(xb.x, xb.y, xb.z, P);
    __shared__ uint32_t staged[8 * kBlock];
    const uint32_t stride = P.boundary_count;
    uint32_t n = 0;
    for_each_neighbour(b.cells, c, P, [&](uint32_t j) {
        const float4 o = __ldg(&b.pos[j]);
        if (dist2(xb.x - o.x, xb.y - o.y, xb.z - o.z) <= P.list_r2) {
            if (n < P.bfl_cap) list_append(b.bfl, k, stride, staged, n, j);
            ++n;
        }
    });
    list_finish(b.bfl, k, stride, staged, n, P.bfl_cap);
    b.bfl_count[k] = n;
}

__global__ void __launch_bounds__(kBlock) k_boundary_cell_bounds(DevParams P, const float4* __restrict__ b_pos,
                                                                 int* __restrict__ bounds) {
    const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
    if (k >= P.boundary_count) return;
    const float4 xb = b_pos[k];
    const Cell c = cell_of(xb.x, xb.y, xb.z, P);
    const int v[3] = {(int)c.x, (int)c.y, (int)c.z};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int lo = __reduce_min_sync(__activemask(), v[a]), hi = __reduce_max_sync(__activemask(), v[a]);
        if ((threadIdx.x & 31) == __ffs(__activemask()) - 1) {
            atomicMin(&bounds[a], lo);
            atomicMax(&bounds[3 + a], hi);
        }
    }
}

// Mark every cell within two cells (each axis) of boundary particle k's cell; the box org + [0, dim) holds
// them all (the boundary's cell bounds widened by two).
__global__ void __launch_bounds__(kBlock) k_boundary_zone(DevParams P, const float4* __restrict__ b_pos, int ox,
                                                          int oy, int oz, uint32_t nx, uint32_t ny,
                                                          unsigned char* __restrict__ zone) {
    const uint32_t k = blockIdx.x * kBlock + threadIdx.x;
    if (k >= P.boundary_count) return;
    const float4 xb = b_pos[k];
    const Cell c = cell_of(xb.x, xb.y, xb.z, P);
    const uint32_t x0 = (uint32_t)((int)c.x - ox) - 2u, y0 = (uint32_t)((int)c.y - oy) - 2u,
                   z0 = (uint32_t)((int)c.z - oz) - 2u;
#pragma unroll 1
    for (uint32_t dz = 0; dz < 5; ++dz)
#pragma unroll 1
        for (uint32_t dy = 0; dy < 5; ++dy)
#pragma unroll
            for (uint32_t dx = 0; dx < 5; ++dx)
                zone[((size_t)(z0 + dz) * ny + (y0 + dy)) * nx + (x0 + dx)] = 1;
}

// pcisph.cl:212-263 with boundary_update = 1 from boundary particle k's fluid list: a fluid particle not
// listed was farther than r_list from x_b at the step's start, so it is farther than h from x_b at its
// prediction unless it moved more than half the skin, which flags its bucket (then k walks).
template <bool kCoherent = false>
__device__ __forceinline__ void boundary_pressure_list_body(const DevParams& P, const Control* ctl,
                                                            const ListBuffers& b, uint32_t k) {
    if (k >= P.boundary_count) return;
    const float4 xb = b.b_pos[k];
    float acc = b.b_init[k];
    const uint32_t cnt = b.bfl_count[k];
    bool walk = cnt > P.bfl_cap;
    Cell c{0u, 0u, 0u};
    if (walk || ctl->fast_particles != ctl->fast_at_begin) {
        c = cell_of(xb.x, xb.y, xb.z, P);
        walk = walk || near_fast(P, b.bucket_fast, c);
    }
    auto f = [&](uint32_t j) { boundary_density_term(xb, load_slot<kCoherent>(&b.pred[j]), P.h2, acc); };
    if (walk) for_each_neighbour(b.cells, c, P, f);
    else for_each_listed(b.bfl, k, cnt, P.boundary_count, f);
    boundary_pressure_finish(P, xb, acc, b.b_press, const_cast<float4*>(b.bpf), k);
}

__global__ void __launch_bounds__(kBlock) k_boundary_pressure_list(DevParams P, const Control* ctl, ListBuffers b) {
    boundary_pressure_list_body(P, ctl, b, blockIdx.x * kBlock + threadIdx.x);
}

// pcisph.cl:65-92, and the neighbour list of the step. kBoundary: the scene has boundary particles (their
// walk and list are compiled out otherwise: the fluid-only builder measured 5% slower with them present)
template <class PS, bool kBoundary>
// (at most 40 registers: 6 blocks, 48 warps per SM; 46 registers measured 5% slower at 1M)
__global__ void __launch_bounds__(kBlock, 6) k_density_list(PS ps, ListBuffers b) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= ps.count()) return;
    const DevParams& P = ps.params(i);
    const float4 xi = b.pos[i];  // xi.w: the particle's stored half skin
    const Cell c = cell_of(xi.x, xi.y, xi.z, P);
    const float sh_i = half_skin_of(P, xi.w);
    const float list_r2 = particle_list_r2(P, sh_i), blist_r2 = boundary_list_r2(P, sh_i);
    float acc = 0.f;
    const uint32_t stride = b.nbr_stride;
    // current chunk of each thread's skin and within-h lists; the boundary list's chunks go through the
    // within-h buffer before the fluid walk starts (more shared memory would take it from the L1 cache)
    __shared__ uint32_t staged[2][8 * kBlock];
    uint32_t* fbuf = staged[0];
    uint32_t* nbuf = staged[1];
    if (kBoundary && P.boundary_count && b.b_zone && !in_boundary_zone(b, c)) {
        b.b_near[i] = 0;  // every boundary particle is at least 2h away
        if (b.bnbr) b.bnbr_count[i] = 0;
    } else if (kBoundary && P.boundary_count) {
        // boundary particles within r_list, in walk order: the later sweeps read them from the boundary list
        // (all of them, or walk the boundary buckets when there are more than bnd_cap)
        uint32_t nb = 0;
        uint32_t* bbuf = staged[1];
        for_each_neighbour(b.b_cells, c, P, [&](uint32_t j) {
            const float4 o = __ldg(&b.b_pos[j]);
            const float r2 = dist2(xi.x - o.x, xi.y - o.y, xi.z - o.z);
            acc += poly6(r2, P.h2);  // density_term's expression
            if (r2 <= blist_r2) {
                if (b.bnbr && nb < P.bnd_cap) list_append(b.bnbr, i, stride, bbuf, nb, j);
                ++nb;
            }
        });
        b.b_near[i] = nb ? 1 : 0;
        if (b.bnbr) {
            list_finish(b.bnbr, i, stride, bbuf, nb, P.bnd_cap);
            b.bnbr_count[i] = nb;
        }
    }
    uint32_t n = 0, nn = 0;
    auto load = [&](uint32_t j) { return __ldg(&b.pos[j]); };
    auto use = [&](uint32_t j, const float4& o) {
        const float dx = xi.x - o.x, dy = xi.y - o.y, dz = xi.z - o.z;
        const float r2 = dist2(dx, dy, dz);
        acc += poly6(r2, P.h2);
        if (r2 <= list_r2) {
            if (n < P.list_cap) list_append(b.nbr, i, stride, fbuf, n, j);
            ++n;
            if (r2 <= P.near_r2) {
                if (nn < P.near_cap) list_append(b.near, i, stride, nbuf, nn, j);
                ++nn;
            }
        }
    };
    for_each_neighbour_prefetched(b.cells, c, P, load, use);
    list_finish(b.nbr, i, stride, fbuf, n, P.list_cap);
    list_finish(b.near, i, stride, nbuf, nn, P.near_cap);
    b.nbr_count[i] = n;  // n > list_cap: this particle walks the buckets in the pressure sweeps
    b.near_count[i] = nn;  // nn > near_cap: it walks them in the sweeps at the current positions
    acc *= P.particle_mass * P.poly6_norm;
    b.rho[i] = acc;
    b.pr4[i] = make_float4(xi.x, xi.y, xi.z, acc);
}

// pcisph.cl:94-112
template <class PS>
__global__ void __launch_bounds__(kBlock) k_normal_list(PS ps, ListBuffers b) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= ps.count()) return;
    const DevParams& P = ps.params(i);
    const float4 xi = b.pr4[i];
    float3 n = make_float3(0.f, 0.f, 0.f);
    const uint32_t cnt = b.near_count[i];
    auto f = [&](uint32_t j) { normal_term(xi.x, xi.y, xi.z, __ldg(&b.pr4[j]), P.h2, n); };
    if (cnt <= P.near_cap) for_each_listed(b.near, i, cnt, b.nbr_stride, f);
    else for_each_neighbour(b.cells, cell_of(xi.x, xi.y, xi.z, P), P, f);
    const float scale = P.h * P.particle_mass * P.poly6_d1_norm;
    b.normal[i] = make_float4(n.x * scale, n.y * scale, n.z * scale, 0.f);
}

// pcisph.cl:121-173, then the first predict (pcisph.cl:175-193, F_p = 0)
template <class PS>
__global__ void __launch_bounds__(kBlock) k_force_list(PS ps, ListBuffers b) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= ps.count()) return;
    const DevParams& P = ps.params(i);
    const float4 xi = b.pr4[i];
    const float3 vi = f3(b.vel[i]);
    const float3 ni = f3(b.normal[i]);
    ForceAccum fa{make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f), make_float3(0.f, 0.f, 0.f)};
    const uint32_t cnt = b.near_count[i];
    auto f = [&](uint32_t j) {
        force_term(xi, vi, ni, __ldg(&b.pr4[j]), f3(__ldg(&b.vel[j])), f3(__ldg(&b.normal[j])), P, fa);
    };
    if (cnt <= P.near_cap) for_each_listed(b.near, i, cnt, b.nbr_stride, f);
    else for_each_neighbour(b.cells, cell_of(xi.x, xi.y, xi.z, P), P, f);
    const float m = P.particle_mass;
    const float3 fo = other_force(m, P.gravity, fa.visc, P.viscosity * m * P.visc_d2_norm, fa.coh,
                                  -P.st_coeff * m * m * P.st_norm, fa.curv, -P.st_coeff * m);
    b.f_other[i] = f4(fo, 0.f);
    b.press[i] = 0.f;
    const float3 v = vi + (fo / m) * P.dt;
    const float3 dx = v * P.dt;
    const float4 xs = make_float4(xi.x + dx.x, xi.y + dx.y, xi.z + dx.z, 0.f);
    b.pred[i] = xs;
    const float disp = note_displacement(P, ps.control(i), b.bucket_fast, xi, xs, P.list_half_skin,
                                         PS::kBatched ? nullptr : b.fast_list, i);
    if (P.particle_skin) b.disp_max[i] = disp;
}

// Partner marks after a prediction round (one scene). A pair of the reference's walk whose predictions are
// within h is in the skin list unless one of the two predictions is fast (moved more than half the skin), so
// the pressure sweep of particle i can use its list unless i is fast or some fast j has x*_j within h of
// x*_i while j is not in i's list. For every fast j of the round (the fast list), thread (j, o) takes cell o
// of the 5 x 5 x 5 cells around x*_j's cell: a particle i that is not fast lies within
// D = h + skin_max_half (< 2 cells, checked on the host) of x*_j, so its cell is among them, and only the
// cells whose box comes within D of x*_j (with a margin for the divisions of cell_of) are scanned. It stamps i
// with the round's number when |x*_i - x*_j| <= h (the pressure sweep's |d|^2, with d negated: the same bits)
// and |x_i - x_j| is beyond i's list radius (the builder's test, the same bits), and stamps j itself.
// Stamping more than needed only makes a particle walk, which gives the walk's sum. The round is the one the
// next pressure sweep reads (Control::round + 1); that sweep's last block closes it. A round with more than
// mark_cap fast predictions stamps nothing (the sweep then uses the bucket flags).
__global__ void __launch_bounds__(kBlock) k_mark_partners(DevParams P, const Control* ctl, ListBuffers b) {
    const unsigned long long n = ctl->fast_n;
    if (n == 0 || n > P.mark_cap) return;
    const unsigned round = ctl->round + 1u;
    const float reach = P.h + P.skin_max_half + 0.01f * P.cell_size;
    const unsigned long long items = n * 125ull;
    for (unsigned long long t = (unsigned long long)blockIdx.x * kBlock + threadIdx.x; t < items;
         t += (unsigned long long)gridDim.x * kBlock) {
        const uint32_t j = b.fast_list[t / 125ull];
        const uint32_t o = (uint32_t)(t % 125ull);
        if (o == 62u) b.walk_stamp[j] = round;  // the centre cell's thread: j itself walks
        const float4 pj = b.pred[j];
        const float4 xj = b.pos[j];
        const Cell c0 = cell_of(pj.x, pj.y, pj.z, P);
        const int off[3] = {(int)(o % 5u) - 2, (int)(o / 5u % 5u) - 2, (int)(o / 25u) - 2};
        const uint32_t cc[3] = {c0.x + (uint32_t)off[0], c0.y + (uint32_t)off[1], c0.z + (uint32_t)off[2]};
        // Skip a cell whose box is farther than the reach from x*_j. Within 2^14 cells of the origin the
        // rounding of the box bounds and of cell_of's division is far below the margin in the reach; farther
        // out (or saturated, or NaN) every cell is scanned.
        auto inner = [](uint32_t c) { return c + 16384u < 32768u; };  // -2^14 < (int)c < 2^14, wrapping
        if (inner(c0.x) && inner(c0.y) && inner(c0.z)) {
            const float pc[3] = {pj.x, pj.y, pj.z};
            float gap2 = 0.f;  // squared distance from x*_j to the cell's box
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const float lo = (float)(int)cc[a] * P.cell_size, hi = lo + P.cell_size;
                const float g = fmaxf(fmaxf(lo - pc[a], pc[a] - hi), 0.f);
                gap2 += g * g;
            }
            if (gap2 > reach * reach) continue;
        }
        const uint2 r = b.cells[P.bucket_base + hash_key(cc[0], cc[1], cc[2], P)];
#pragma unroll 1
        for (uint32_t i0 = r.x; i0 < r.y; i0 += 4) {
            float4 pi[4], xi[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i0 + u < r.y) {
                    pi[u] = b.pred[i0 + u];
                    xi[u] = b.pos[i0 + u];
                }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (i0 + u < r.y && dist2(pj.x - pi[u].x, pj.y - pi[u].y, pj.z - pi[u].z) <= P.h2 &&
                    !(dist2(xi[u].x - xj.x, xi[u].y - xj.y, xi[u].z - xj.z) <=
                      particle_list_r2(P, half_skin_of(P, xi[u].w))))
                    b.walk_stamp[i0 + u] = round;
        }
    }
}

// pcisph.cl:212-263 (boundary_update = 0); one scene: also the stop decision in the last block
// One particle's pressure sweep; returns its density variation (0 when skipped or out of range).
template <class PS, bool kCoherent = false>
__device__ __forceinline__ float pressure_body(const PS& ps, const ListBuffers& b, uint32_t i) {
    float dv = 0.f;
    if (i < ps.count() && !ps.skip_pressure(i)) {
        const DevParams& P = ps.params(i);
        Control* ctl = ps.control(i);
        // no particle of the scene moved more than half the skin: its lists are complete for x*
        const bool all_lists_ok = ctl->fast_particles == ctl->fast_at_begin;
        const float4 xi = b.pos[i];
        const float4 xp = b.pred[i];
        float acc = 0.f;
        const uint32_t cnt = b.nbr_count[i];
        const bool overflow = cnt > P.list_cap;
        // self_fast: x* moved more than the particle's own half skin from x, so its lists (built for that
        // skin) may miss a pair: with per-particle skins it walks. Boundary terms: all zero unless a boundary
        // particle was within r_list of x, or x* moved past the half skin (boundary particles do not move);
        // within it, the boundary list (every boundary particle within r_list of x) holds every one that can
        // be within h of x*.
        bool self_fast = false;
        if (P.particle_skin || P.boundary_count) {
            const float dx = xp.x - xi.x, dy = xp.y - xi.y, dz = xp.z - xi.z;
            self_fast = sqrtf(dist2(dx, dy, dz)) > fast_threshold(P, half_skin_of(P, xi.w));
        }
        bool walk_boundary = false, list_boundary = false;
        uint32_t bcnt = 0;
        if (P.boundary_count) {
            if (self_fast) {
                walk_boundary = true;
            } else if (b.b_near[i] != 0) {
                if (b.bnbr) bcnt = b.bnbr_count[i];
                list_boundary = b.bnbr && bcnt <= P.bnd_cap;
                walk_boundary = !list_boundary;
            }
        }
        Cell c{0u, 0u, 0u};  // the cell (three IEEE divisions) only where a walk may need it
        const bool own_walk = overflow || (P.particle_skin && self_fast);
        // partner marks of this round (one scene, after the marking kernel): the particles that may miss a
        // pair of their walk are stamped with the round's number; a round past the cap (or no marks) takes
        // the bucket flags: every particle near a fast one walks
        const unsigned long long fast_round = !PS::kBatched && b.walk_stamp ? ctl->fast_n : ~0ull;
        const bool marks = fast_round <= P.mark_cap;
        bool walk;
        if (marks) {
            walk = own_walk || (fast_round != 0 && b.walk_stamp[i] == ctl->round + 1u);
            if (walk || walk_boundary) c = cell_of(xi.x, xi.y, xi.z, P);
        } else {
            if (own_walk || !all_lists_ok || walk_boundary) c = cell_of(xi.x, xi.y, xi.z, P);
            walk = own_walk || (!all_lists_ok && near_fast(P, b.bucket_fast, c));
        }
        auto fb = [&](uint32_t j) { acc += density_term(xp.x, xp.y, xp.z, __ldg(&b.b_pos[j]), P.h2); };
        if (walk_boundary) for_each_neighbour(b.b_cells, c, P, fb);
        else if (list_boundary) for_each_listed(b.bnbr, i, bcnt, b.nbr_stride, fb);
        auto f = [&](uint32_t j) { acc += density_term(xp.x, xp.y, xp.z, load_slot<kCoherent>(&b.pred[j]), P.h2); };
        if (walk) {
            // a batch walks with two gathers in flight (terms still added in walk order): its walkers are
            // few and latency-bound (256 batched scenes, 9.8M particles, over 500 steps: 26.8 -> 25.8 s); one scene walks plainly
            // (8M particles all walking: 3.0 ms per sweep, 3.6 with the prefetch)
            if constexpr (PS::kBatched)
                for_each_neighbour_prefetched(
                    b.cells, c, P, [&](uint32_t j) { return load_slot<kCoherent>(&b.pred[j]); },
                    [&](uint32_t, const float4& o) { acc += density_term(xp.x, xp.y, xp.z, o, P.h2); });
            else
                for_each_neighbour(b.cells, c, P, f);
        } else {
            for_each_listed(b.nbr, i, cnt, b.nbr_stride, f);
        }
        acc *= P.particle_mass * P.poly6_norm;
        if (!isfinite(acc)) atomicOr(&ctl->status, 2u);
        dv = acc - P.rest_density;
        dv = 0.f < dv ? dv : 0.f;
        b.err[i] = dv;
        float p = b.press[i];
        if (dv != 0.f) {
            p += dv * P.delta;
            b.press[i] = p;
        }
        const float r = b.rho[i];
        b.pf4[i] = make_float4(xi.x, xi.y, xi.z, p / (r * r));
        if (PS::kBatched) warp_atomic_max(&ctl->max_err_bits, __float_as_uint(dv));
    }
    return dv;
}

// BS: threads per block (128, 256 or 512; the autotuner's choice for one scene)
template <class PS, int BS = kBlock>
__global__ void __launch_bounds__(BS) k_pressure_list(PS ps, ListBuffers b) {
    const float dv = pressure_body(ps, b, blockIdx.x * BS + threadIdx.x);
    if (PS::kBatched) return;
    // one scene: block max of dv, the last block decides (dv >= 0: bit patterns order like values)
    const unsigned bits = __reduce_max_sync(0xffffffffu, __float_as_uint(dv));
    __shared__ unsigned warp_max[BS / 32];
    __shared__ bool is_last;
    if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = bits;
    __syncthreads();
    Control* ctl = ps.control(0);
    if (threadIdx.x == 0) {
        unsigned m = 0;
#pragma unroll
        for (int w = 0; w < BS / 32; ++w) m = max(m, warp_max[w]);
        atomicMax(&ctl->max_err_bits, m);
        __threadfence();
        is_last = atomicAdd(&ctl->blocks_done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (is_last && threadIdx.x == 0) {
        __threadfence();
        ctl->max_err_bits = atomicAdd(&ctl->max_err_bits, 0u);  // see every block's contribution
        if (b.walk_stamp) {  // close the prediction round of the partner marks: the next one starts empty
            ctl->round += 1u;
            ctl->fast_n = 0;
        }
        decide(ps.params(0), ctl);
    }
}

// pcisph.cl:265-300, then predict (pcisph.cl:175-193) or integrate with optional walls
// One particle's pressure-force sweep, then predict (mode 0 before the decision, 1) or integrate (mode 0
// after it, 2) with optional walls.
template <class PS, bool kCoherent = false>
__device__ __forceinline__ void pressure_force_body(const PS& ps, const ListBuffers& b, uint32_t i, int mode) {
    if (i >= ps.count() || ps.skip_force(i)) return;
    const DevParams& P = ps.params(i);
    Control* ctl = ps.control(i);
    const float4 xi = b.pf4[i];
    float3 f = make_float3(0.f, 0.f, 0.f);
    const uint32_t cnt = b.near_count[i];
    // boundary terms at x (within h): all zero unless a boundary particle was within r_list of x; the
    // boundary list holds every one within r_list (terms beyond h are zero)
    const bool near_b = P.boundary_count && b.b_near[i] != 0;
    const uint32_t bcnt = near_b && b.bnbr ? b.bnbr_count[i] : 0u;
    const bool list_boundary = near_b && b.bnbr && bcnt <= P.bnd_cap;
    const bool walk_boundary = near_b && !list_boundary;
    Cell c{0u, 0u, 0u};
    if (cnt > P.near_cap || walk_boundary) c = cell_of(xi.x, xi.y, xi.z, P);
    auto fb = [&](uint32_t j) { pressure_force_term(xi, load_slot<kCoherent>(&b.bpf[j]), P.h, P.h2, f); };
    if (walk_boundary) for_each_neighbour(b.b_cells, c, P, fb);
    else if (list_boundary) for_each_listed(b.bnbr, i, bcnt, b.nbr_stride, fb);
    auto body = [&](uint32_t j) { pressure_force_term(xi, load_slot<kCoherent>(&b.pf4[j]), P.h, P.h2, f); };
    if (cnt <= P.near_cap) for_each_listed(b.near, i, cnt, b.nbr_stride, body);
    else for_each_neighbour(b.cells, c, P, body);
    const float m = P.particle_mass;
    const float scale = -P.spiky_d1_norm * m * m;
    const float3 fp = make_float3(f.x * scale, f.y * scale, f.z * scale);
    b.f_press[i] = f4(fp, 0.f);
    const bool integrate = mode == 0 ? (ctl->done != 0u) : mode == 2;
    const float3 a = (f3(b.f_other[i]) + fp) / m;
    float3 v = f3(b.vel[i]) + a * P.dt;
    const float3 dx = v * P.dt;
    float3 x = make_float3(xi.x + dx.x, xi.y + dx.y, xi.z + dx.z);
    if (!integrate) {
        const float4 xs = f4(x, 0.f);
        b.pred[i] = xs;
        const float disp = note_displacement(P, ctl, b.bucket_fast, xi, xs, P.list_half_skin,
                                             PS::kBatched ? nullptr : b.fast_list, i);
        if (P.particle_skin) b.disp_max[i] = fmaxf(b.disp_max[i], disp);
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
    const uint32_t o = b.out_index ? b.out_index[i] : i;  // working order -> sorted order
    b.state_pos[o] = f4(x, 0.f);
    b.state_vel[o] = f4(v, 0.f);
    if (P.particle_skin)  // the next step's half skin: twice this step's largest predicted displacement
        b.state_skin[o] = fminf(fmaxf(P.skin_factor * b.disp_max[i], P.skin_min_half), P.skin_max_half);
}

template <class PS, int BS = kBlock>
// (at most 40 registers: 48 resident warps per SM; 48 registers measured 10% slower at 1M)
__global__ void __launch_bounds__(BS, 1536 / BS) k_pressure_force_list(PS ps, ListBuffers b, int mode,
                                                            cudaGraphConditionalHandle cond, int use_cond) {
    const uint32_t i = blockIdx.x * BS + threadIdx.x;
    if (!PS::kBatched && use_cond && i == 0) {
        // continue the graph's while loop unless the step is done; the counter bounds it on its own
        Control* ctl = ps.control(0);
        const unsigned g = ++ctl->guard_iters;
        const bool stop = ctl->done != 0u || g >= (unsigned)ps.params(0).max_iters;
        cudaGraphSetConditional(cond, stop ? 0u : 1u);
    }
    pressure_force_body(ps, b, i, mode);
}

// The corrective loop of one step as one cooperative launch (every block resident, grid-stride over the
// particles): pressure sweep, grid barrier, the loop decision in block 0 (one scene, or every scene of a
// batch with its own convergence flags), grid barrier, pressure-force sweep, grid barrier; until no scene
// iterates, at most max_iters times. Same sweeps and decisions as the graph's while loop, so the same bits.
// Every thread takes every barrier: the bodies return to the loop, never out of the kernel.
template <class PS>
__global__ void __launch_bounds__(kBlock) k_corrective_loop(PS ps, ListBuffers b, Control* loop, int max_iters) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    const uint32_t stride = gridDim.x * kBlock;
    const uint32_t rounds = (ps.count() + stride - 1) / stride;
    __shared__ int running;
    for (int it = 0; it < max_iters; ++it) {
        if constexpr (!PS::kBatched) {  // boundary pressures at the predicted positions (read by the force)
            const DevParams& P = ps.params(0);
            for (uint32_t k = blockIdx.x * kBlock + threadIdx.x; k < P.boundary_count; k += stride)
                boundary_pressure_list_body<true>(P, ps.control(0), b, k);
        }
        unsigned local = 0;
        for (uint32_t r = 0; r < rounds; ++r)
            local = max(local, __float_as_uint(
                                   pressure_body<PS, true>(ps, b, r * stride + blockIdx.x * kBlock + threadIdx.x)));
        if (!PS::kBatched) {  // batched scenes reduced per scene inside the body
            const unsigned m = __reduce_max_sync(0xffffffffu, local);
            if ((threadIdx.x & 31) == 0 && m) atomicMax(&ps.control(0)->max_err_bits, m);
        }
        grid.sync();
        if (blockIdx.x == 0) {
            if (threadIdx.x == 0) running = 0;
            __syncthreads();
            if constexpr (!PS::kBatched) {
                if (threadIdx.x == 0) {
                    Control* c = ps.control(0);
                    decide(ps.params(0), c);
                    running = c->done ? 0 : 1;
                }
            } else {
                for (uint32_t sc = threadIdx.x; sc < ps.n_scenes; sc += blockDim.x) {
                    Control* c = &ps.ctls[sc];
                    if (c->done) {
                        c->finished = 1;
                        continue;
                    }
                    decide(ps.table[sc], c);
                    if (!c->done) atomicOr(&running, 1);
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                loop->guard_iters += 1;
                if (PS::kBatched) loop->total_iters += 1;
                loop->any_running = running ? 1u : 0u;
            }
        }
        grid.sync();
        for (uint32_t r = 0; r < rounds; ++r)
            pressure_force_body<PS, true>(ps, b, r * stride + blockIdx.x * kBlock + threadIdx.x, 0);
        grid.sync();
        if (*reinterpret_cast<volatile unsigned*>(&loop->any_running) == 0u) break;
    }
}

// Batch: close one corrective iteration per scene (one thread per scene) and set the graph's loop
// condition: continue while some scene iterates. A scene decided done here is integrated by the
// pressure-force sweep that follows; the next call marks it finished. Every scene is done by its
// max_iters, so the loop ends; the guard bounds it by the largest max_iters on its own.
__global__ void k_batch_decide(const DevParams* __restrict__ table, Control* ctls, uint32_t n_scenes, Control* batch,
                               int max_iters, cudaGraphConditionalHandle cond, int use_cond) {
    __shared__ int running;
    if (threadIdx.x == 0) running = 0;
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < n_scenes; s += blockDim.x) {
        Control* c = &ctls[s];
        if (c->done) {
            c->finished = 1;
            continue;
        }
        decide(table[s], c);
        if (!c->done) atomicOr(&running, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned g = ++batch->guard_iters;
        batch->total_iters += 1;
        const bool more = running != 0 && g < (unsigned)max_iters;
        batch->any_running = more ? 1u : 0u;
        if (use_cond) cudaGraphSetConditional(cond, more ? 1u : 0u);
    }
}

// Batch step start: per-scene iteration state.
// Per scene, before a step: reset the step's control fields. A scene with an adaptive skin takes the
// smallest skin level that at most 1 in skin_outrun_ratio of the previous step's predictions outran (the
// largest if none), from that step's counts, and writes its list radius into the scene table; the builder
// and the sweeps of this step read it there. Results do not depend on the choice.
__global__ void k_batch_begin(DevParams* table, Control* ctls, uint32_t n_scenes, Control* batch) {
    for (uint32_t s = threadIdx.x; s < n_scenes; s += blockDim.x) {
        Control* c = &ctls[s];
        DevParams* P = &table[s];
        if (P->adaptive_skin) {
            int level = 0;
            if (c->steps) {
                const unsigned long long preds =
                    (unsigned long long)P->fluid_count * (unsigned long long)max(c->iterations_last, 1);
                level = kSkinLevels - 1;
                for (int k = kSkinLevels - 1; k >= 0; --k)
                    if (c->over_level[k] * (unsigned long long)P->skin_outrun_ratio <= preds) level = k;
            }
            c->skin_level = (unsigned)level;
            set_list_skin(P, skin_level_value(level));
            for (int k = 0; k < kSkinLevels; ++k) c->over_level[k] = 0;
        }
        c->iter = 0;
        c->done = 0;
        c->finished = 0;
        c->max_err_bits = 0;
        c->fast_at_begin = c->fast_particles;
        c->status = 0;
    }
    if (threadIdx.x == 0) {
        batch->guard_iters = 0;
        batch->any_running = 1;
        batch->status = 0;  // the reorder flags an out-of-range sorted index here
    }
}

__global__ void __launch_bounds__(kBlock) k_scene_of(const uint32_t* __restrict__ offsets, uint32_t n_scenes,
                                                     uint32_t n, uint16_t* __restrict__ scene_of) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    uint32_t lo = 0, hi = n_scenes;  // largest s with offsets[s] <= i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (offsets[mid] <= i) lo = mid;
        else hi = mid;
    }
    scene_of[i] = (uint16_t)lo;
}

// sort_utils.cl:12-23 per scene, offset into the scene's bucket range of the shared table
__global__ void __launch_bounds__(kBlock) k_hash_scenes(SceneTable ps, const float4* __restrict__ pos,
                                                        uint32_t* __restrict__ keys) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= ps.count()) return;
    const DevParams& P = ps.params(i);
    const float4 p = pos[i];
    const Cell c = cell_of(p.x, p.y, p.z, P);
    keys[i] = P.bucket_base + hash_key(c.x, c.y, c.z, P);
}

}  // namespace

void launch_density_list(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s) {
    if (P.boundary_count) k_density_list<OneScene, true><<<grid_for(P.fluid_count), kBlock, 0, s>>>(OneScene{P, ctl}, b);
    else k_density_list<OneScene, false><<<grid_for(P.fluid_count), kBlock, 0, s>>>(OneScene{P, ctl}, b);
}
void launch_normal_list(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s) {
    k_normal_list<<<grid_for(P.fluid_count), kBlock, 0, s>>>(OneScene{P, ctl}, b);
}
void launch_force_list(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s) {
    k_force_list<<<grid_for(P.fluid_count), kBlock, 0, s>>>(OneScene{P, ctl}, b);
}
void launch_pressure_list(const DevParams& P, Control* ctl, const ListBuffers& b, int block, cudaStream_t s) {
    const OneScene ps{P, ctl};
    const uint32_t n = P.fluid_count;
    if (block == 128) k_pressure_list<OneScene, 128><<<(n + 127) / 128, 128, 0, s>>>(ps, b);
    else if (block == 512) k_pressure_list<OneScene, 512><<<(n + 511) / 512, 512, 0, s>>>(ps, b);
    else k_pressure_list<OneScene, kBlock><<<grid_for(n), kBlock, 0, s>>>(ps, b);
}
void launch_mark_partners(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s) {
    k_mark_partners<<<kMarkBlocks, kBlock, 0, s>>>(P, ctl, b);
}
void launch_pressure_force_list(const DevParams& P, Control* ctl, const ListBuffers& b, int mode,
                                cudaGraphConditionalHandle cond, bool use_cond, int block, cudaStream_t s) {
    const OneScene ps{P, ctl};
    const uint32_t n = P.fluid_count;
    const int uc = use_cond ? 1 : 0;
    if (block == 128) k_pressure_force_list<OneScene, 128><<<(n + 127) / 128, 128, 0, s>>>(ps, b, mode, cond, uc);
    else if (block == 512) k_pressure_force_list<OneScene, 512><<<(n + 511) / 512, 512, 0, s>>>(ps, b, mode, cond, uc);
    else k_pressure_force_list<OneScene, kBlock><<<grid_for(n), kBlock, 0, s>>>(ps, b, mode, cond, uc);
}

namespace {
template <class PS>
cudaError_t launch_loop(const PS& ps, uint32_t n, const ListBuffers& b, Control* loop, int max_iters, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_corrective_loop<PS>, kBlock, 0);
    if (e != cudaSuccess) return e;
    if (!coop || per_sm < 1) return cudaErrorNotSupported;
    const unsigned blocks = std::min<unsigned>((unsigned)(sms * per_sm), grid_for(n));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kBlock);
    cfg.stream = s;
    cudaLaunchAttribute attr{};
    attr.id = cudaLaunchAttributeCooperative;
    attr.val.cooperative = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_corrective_loop<PS>, ps, b, loop, max_iters);
}
}  // namespace

cudaError_t launch_corrective_loop(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s) {
    return launch_loop(OneScene{P, ctl}, P.fluid_count, b, ctl, P.max_iters, s);
}
cudaError_t launch_corrective_loop_scenes(const SceneTable& t, const ListBuffers& b, Control* batch, int max_iters,
                                          cudaStream_t s) {
    return launch_loop(t, t.n, b, batch, max_iters, s);
}

void launch_boundary_cell_bounds(const DevParams& P, const float4* b_pos, int* bounds, cudaStream_t s) {
    if (P.boundary_count) k_boundary_cell_bounds<<<grid_for(P.boundary_count), kBlock, 0, s>>>(P, b_pos, bounds);
}
void launch_boundary_zone(const DevParams& P, const float4* b_pos, const int* org, const uint32_t* dim,
                          unsigned char* zone, cudaStream_t s) {
    if (P.boundary_count)
        k_boundary_zone<<<grid_for(P.boundary_count), kBlock, 0, s>>>(P, b_pos, org[0], org[1], org[2], dim[0],
                                                                      dim[1], zone);
}
void launch_boundary_fluid_list(const DevParams& P, const ListBuffers& b, cudaStream_t s) {
    if (P.boundary_count) k_boundary_fluid_list<<<grid_for(P.boundary_count), kBlock, 0, s>>>(P, b);
}
void launch_boundary_pressure_list(const DevParams& P, Control* ctl, const ListBuffers& b, cudaStream_t s) {
    if (P.boundary_count) k_boundary_pressure_list<<<grid_for(P.boundary_count), kBlock, 0, s>>>(P, ctl, b);
}
void launch_batch_begin(DevParams* table, Control* ctls, uint32_t n_scenes, Control* batch, cudaStream_t s) {
    k_batch_begin<<<1, 256, 0, s>>>(table, ctls, n_scenes, batch);
}
void launch_scene_of(const uint32_t* offsets, uint32_t n_scenes, uint32_t n, uint16_t* scene_of, cudaStream_t s) {
    if (n) k_scene_of<<<grid_for(n), kBlock, 0, s>>>(offsets, n_scenes, n, scene_of);
}
void launch_hash_scenes(const SceneTable& t, const float4* pos, uint32_t* keys, cudaStream_t s) {
    if (t.n) k_hash_scenes<<<grid_for(t.n), kBlock, 0, s>>>(t, pos, keys);
}
void launch_density_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s) {
    if (t.n) k_density_list<SceneTable, false><<<grid_for(t.n), kBlock, 0, s>>>(t, b);  // no boundary in a batch
}
void launch_normal_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s) {
    if (t.n) k_normal_list<<<grid_for(t.n), kBlock, 0, s>>>(t, b);
}
void launch_force_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s) {
    if (t.n) k_force_list<<<grid_for(t.n), kBlock, 0, s>>>(t, b);
}
void launch_pressure_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s) {
    if (t.n) k_pressure_list<<<grid_for(t.n), kBlock, 0, s>>>(t, b);
}
void launch_pressure_force_scenes(const SceneTable& t, const ListBuffers& b, cudaStream_t s) {
    if (t.n) k_pressure_force_list<<<grid_for(t.n), kBlock, 0, s>>>(t, b, 0, 0, 0);
}
void launch_batch_decide(const SceneTable& t, Control* batch, int max_iters, cudaGraphConditionalHandle cond,
                         bool use_cond, cudaStream_t s) {
    k_batch_decide<<<1, 256, 0, s>>>(t.table, t.ctls, t.n_scenes, batch, max_iters, cond, use_cond ? 1 : 0);
}

}  // namespace pcisph
