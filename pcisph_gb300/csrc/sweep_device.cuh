// sweep_device.cuh -- device helpers of the neighbour-list sweeps (list_kernels.cu): warp-aggregated
// counters, the fast-prediction bookkeeping and the corrective loop's decision.
#pragma once
#include "common.cuh"

namespace pcisph {

// atomicMax aggregated over the lanes of a warp that target the same address (one atomic per address).
__device__ __forceinline__ void warp_atomic_max(unsigned* addr, unsigned v) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, (unsigned long long)addr);
    const unsigned m = __reduce_max_sync(peers, v);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicMax(addr, m);
}

// Add the number of this warp's lanes with pred set to *addr: one atomic per group of lanes sharing addr,
// none when no lane has pred.
__device__ __forceinline__ void warp_count(unsigned long long* addr, bool pred) {
    const unsigned act = __activemask();
    const unsigned set = __ballot_sync(act, pred);
    if (!set) return;
    const unsigned peers = __match_any_sync(act, (unsigned long long)addr);
    const unsigned c = __popc(set & peers);
    if (c && (int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(addr, (unsigned long long)c);
}

// After predicting x*_i (stored as xs): a fast particle (moved more than half the skin) flags its bucket
// and is counted (one atomic per warp that has one; no store otherwise: in a splash most predictions are
// fast, and a flag stored by each of their warps measured slower than the counts alone); the predictions
// past each adaptive skin level are counted. With a fast list (partner marks, one scene), a fast particle
// also takes a slot of the round's list while the round holds at most P.mark_cap of them (one atomic per
// warp that has one; none once the round is past the cap, which then falls back to the bucket flags).
// Returns the displacement |x* - x|; threshold: the particle's fast_threshold.
__device__ __forceinline__ float note_displacement(const DevParams& P, Control* ctl,
                                                   unsigned char* __restrict__ bucket_fast, const float4& xi,
                                                   const float4& xs, float threshold,
                                                   uint32_t* __restrict__ fast_list = nullptr, uint32_t i = 0) {
    const float dx = xs.x - xi.x, dy = xs.y - xi.y, dz = xs.z - xi.z;  // exact: xs and xi are close
    const float disp = sqrtf(dist2(dx, dy, dz));
    const bool fast = disp > threshold;
    warp_count(&ctl->fast_particles, fast);
    if (fast_list) {
        const unsigned act = __activemask();
        const unsigned set = __ballot_sync(act, fast);
        if (set) {
            const int lane = (int)(threadIdx.x & 31), leader = __ffs(set) - 1;
            unsigned long long base = ~0ull;
            if (lane == leader && *(volatile unsigned long long*)&ctl->fast_n <= P.mark_cap)
                base = atomicAdd(&ctl->fast_n, (unsigned long long)__popc(set));
            base = __shfl_sync(act, base, leader);
            if (fast && base != ~0ull) {
                const unsigned long long slot = base + __popc(set & ((1u << lane) - 1u));
                if (slot < P.mark_cap) fast_list[slot] = i;
            }
        }
    }
    if (P.adaptive_skin) {
#pragma unroll
        for (int k = 0; k < kSkinLevels; ++k) warp_count(&ctl->over_level[k], disp > P.skin_half[k]);
    }
    if (fast) {
        const Cell c = cell_of(xi.x, xi.y, xi.z, P);
        bucket_fast[P.bucket_base + hash_key(c.x, c.y, c.z, P)] = 1;
    }
    return disp;
}

// The loop decision of one scene after its pressure sweep (Fluid.cpp:284-306).
__device__ __forceinline__ void decide(const DevParams& P, Control* ctl) {
    const float mx = __uint_as_float(ctl->max_err_bits);
    const unsigned it = ctl->iter + 1;
    const float rel = mx / P.rest_density;
    const bool converged = rel < P.threshold;
    const bool done = it >= (unsigned)P.max_iters || (it >= (unsigned)P.min_iters && converged);
    ctl->iter = it;
    ctl->done = done ? 1u : 0u;
    ctl->max_err_bits = 0;
    ctl->blocks_done = 0;
    if (ctl->fast_particles != ctl->fast_at_begin) ctl->list_fallbacks += 1;
    if (done) close_step(ctl, it, rel, converged);
}

}  // namespace pcisph
