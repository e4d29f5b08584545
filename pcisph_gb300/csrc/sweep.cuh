// sweep.cuh -- warp-per-bucket neighbour sweeps with shared-memory staging.
//
// The particles of one bucket run (same key, contiguous in the sorted arrays)
// are processed by one warp. Runs may mix spatial cells (hash collisions), so
// the warp splits its particles ("selves") into sub-groups of one exact cell
// (floor(x / cell_size), as the reference computes it, grid_utils.cl:9-11).
// For each sub-group:
//   1. lanes 0..26 hash the 27 neighbour cells (grid_utils.cl:68-69 order) and
//      read their boundary and fluid bucket ranges; a warp scan lays the 54
//      ranges end to end (boundary first, then fluid, as pcisph.cl sums them);
//   2. candidates are staged in shared memory, window by window, coalesced
//      within each bucket. A candidate whose cell code differs from the cell the
//      bucket was visited for is a hash-collision particle from a cell at least
//      two cells away; it contributes exactly zero in every reference kernel
//      (all of them cut off at r > h) and is not staged;
//   3. lanes take (self s, slice q) pairs and sum over candidates t = q mod Q;
//      a segmented shuffle reduction combines the Q slices of each self, and the
//      lane that holds the self writes the result (deterministic: no atomics).
// Cell codes pack (x & 1023, y & 1023, z & 1023); equal codes can only alias
// cells 1024 apart, which the distance cut-off then rejects, so the filter
// never drops a particle the reference counts.
#pragma once
#include "common.cuh"

namespace pcisph {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kBoundaryTag = 0x80000000u;

__device__ __forceinline__ uint32_t cell_code(uint32_t x, uint32_t y, uint32_t z) {
    return (x & 1023u) | ((y & 1023u) << 10) | ((z & 1023u) << 20);
}

template <class Cand, int CAP>
struct SweepWarpSmem {
    Cand cand[CAP];
    uint32_t bstart[54];  // 0..26 boundary buckets, 27..53 fluid buckets
    uint32_t boff[55];    // exclusive offsets; boff[54] = total
    uint32_t bcode[27];   // expected cell code of each of the 27 neighbour cells
    uint32_t self_lane[32];
};

struct SweepArgs {
    const uint32_t* groups;      // start index of every bucket run
    const uint32_t* n_groups;    // device count
    const uint32_t* keys;        // sorted keys
    const uint2* cells;          // fluid cell table
    const uint2* b_cells;        // boundary cell table
    const uint32_t* codes;       // fluid cell codes (sorted order)
    const uint32_t* b_codes;     // boundary cell codes
};

// Warp-wide exclusive scan; returns the exclusive prefix, total in *tot.
__device__ __forceinline__ uint32_t warp_exclusive_scan(uint32_t v, uint32_t* tot) {
    const int lane = threadIdx.x & 31;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    *tot = __shfl_sync(kFull, x, 31);
    return x - v;
}

// One sub-group: selves in `same` (lanes of this warp), all in cell (cx, cy, cz).
template <class Op, int CAP>
__device__ __forceinline__ void sweep_subgroup(const DevParams& P, const Op& op, const SweepArgs& A,
                                               SweepWarpSmem<typename Op::Cand, CAP>& sm, unsigned same,
                                               uint32_t cx, uint32_t cy, uint32_t cz,
                                               const typename Op::Self& me, uint32_t self_index,
                                               typename Op::Result& my_result) {
    const int lane = threadIdx.x & 31;
    const bool has_b = P.boundary_count != 0;
    // 1. the 27 neighbour buckets
    uint32_t fs = 0, fl = 0, bs = 0, bl = 0;
    if (lane < 27) {
        const int dx = lane % 3 - 1, dy = (lane / 3) % 3 - 1, dz = lane / 9 - 1;
        const uint32_t x = cx + (uint32_t)dx, y = cy + (uint32_t)dy, z = cz + (uint32_t)dz;
        const uint32_t key = P.bucket_base + hash_key(x, y, z, P);
        const uint2 r = __ldg(&A.cells[key]);
        fs = r.x;
        fl = r.y - r.x;
        if (has_b) {
            const uint2 rb = __ldg(&A.b_cells[key]);
            bs = rb.x;
            bl = rb.y - rb.x;
        }
        sm.bcode[lane] = cell_code(x, y, z);
    }
    uint32_t tb, tf;
    const uint32_t ob = warp_exclusive_scan(bl, &tb);
    const uint32_t of = warp_exclusive_scan(fl, &tf);
    if (lane < 27) {
        sm.bstart[lane] = bs;
        sm.boff[lane] = ob;
        sm.bstart[27 + lane] = fs;
        sm.boff[27 + lane] = tb + of;
    }
    const uint32_t T = tb + tf;
    if (lane == 0) sm.boff[54] = T;
    // ranks of the selves
    const int ns = __popc(same);
    if (same & (1u << lane)) sm.self_lane[__popc(same & ((1u << lane) - 1u))] = lane;
    __syncwarp();
    const int Q = 32 / ns;
    const int s = lane / Q, q = lane - s * Q;
    const bool active = s < ns;
    const typename Op::Self sme = Op::shfl(me, active ? (int)sm.self_lane[s] : 0);
    typename Op::Acc acc;
    Op::zero(acc);
    // 2+3. staged windows
    int b = 0;  // per-lane bucket cursor over raw candidate index t
    for (uint32_t w0 = 0; w0 < T; w0 += CAP) {
        uint32_t kept = 0;
        for (uint32_t base = w0; base < min(T, w0 + CAP); base += 32) {
            const uint32_t t = base + lane;
            bool keep = false;
            uint32_t j = 0;
            bool is_b = false;
            if (t < T && t < w0 + CAP) {
                while (sm.boff[b + 1] <= t) ++b;
                j = sm.bstart[b] + (t - sm.boff[b]);
                is_b = b < 27;
                const uint32_t code = is_b ? __ldg(&A.b_codes[j]) : __ldg(&A.codes[j]);
                keep = code == sm.bcode[is_b ? b : b - 27];
            }
            const unsigned kb = __ballot_sync(kFull, keep);
            if (keep) sm.cand[kept + __popc(kb & ((1u << lane) - 1u))] = is_b ? op.load_boundary(j) : op.load_fluid(j);
            kept += __popc(kb);
        }
        __syncwarp();
        if (active) {
#pragma unroll 4
            for (uint32_t t = q; t < kept; t += Q) op.pair(P, sme, sm.cand[t], acc);
        }
        __syncwarp();
    }
    // segmented reduction over the Q slices of each self
    for (int off = 1; off < Q; off <<= 1) {
        const typename Op::Acc v = Op::shfl_down(acc, off);
        if (q + off < Q) Op::add(acc, v);
    }
    const int my_rank = __popc(same & ((1u << lane) - 1u));
    const typename Op::Acc tot = Op::shfl(acc, (same & (1u << lane)) ? my_rank * Q : 0);
    if (same & (1u << lane)) Op::combine(my_result, op.finish(P, self_index, me, tot));
    __syncwarp();
}

// Persistent grid: each warp takes bucket runs g = warp id, warp id + total warps, ...
template <class Op, int WARPS, int CAP>
__global__ void __launch_bounds__(WARPS * 32) k_sweep(DevParams P, Op op, SweepArgs A) {
    extern __shared__ __align__(16) unsigned char sweep_smem[];
    using Smem = SweepWarpSmem<typename Op::Cand, CAP>;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    Smem& sm = reinterpret_cast<Smem*>(sweep_smem)[warp];
    op.begin(P);
    typename Op::Result res = Op::no_result();
    const uint32_t G = *A.n_groups;
    for (uint32_t g = blockIdx.x * WARPS + warp; g < G; g += gridDim.x * WARPS) {
        const uint32_t start = __ldg(&A.groups[g]);
        const uint32_t key = __ldg(&A.keys[start]);
        if (key >= P.bucket_count) continue;  // reorder flagged it already
        const uint32_t end = __ldg(&A.cells[key]).y;
        for (uint32_t c0 = start; c0 < end; c0 += 32) {
            const uint32_t i = c0 + lane;
            const bool valid = i < end;
            typename Op::Self me = Op::empty_self();
            Cell c{0u, 0u, 0u};
            if (valid) {
                me = op.load_self(i);
                const float3 x = Op::cell_pos(me);
                c = cell_of(x.x, x.y, x.z, P);
            }
            unsigned todo = __ballot_sync(kFull, valid);
            while (todo) {
                const int leader = __ffs(todo) - 1;
                const uint32_t lx = __shfl_sync(kFull, c.x, leader);
                const uint32_t ly = __shfl_sync(kFull, c.y, leader);
                const uint32_t lz = __shfl_sync(kFull, c.z, leader);
                const unsigned same = __ballot_sync(kFull, valid && c.x == lx && c.y == ly && c.z == lz);
                todo &= ~same;
                sweep_subgroup<Op, CAP>(P, op, A, sm, same, lx, ly, lz, me, i, res);
            }
        }
    }
    op.end(P, res);
}

template <class Op, int WARPS, int CAP>
constexpr size_t sweep_smem_bytes() {
    return sizeof(SweepWarpSmem<typename Op::Cand, CAP>) * WARPS;
}

}  // namespace pcisph
