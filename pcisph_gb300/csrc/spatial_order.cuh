// spatial_order.cuh -- the step's working order: the reference's sorted order with whole buckets moved
// into Morton order of their cells (spatial_order.cu).
//
// The reference sorts particles by hash key (sort_utils.cl:12-23) and walks buckets in that "sorted"
// order, so neighbouring cells lie at random places in memory. The working order keeps every bucket
// contiguous and in its sorted internal order but places the buckets by the Morton code of their first
// particle's cell: a warp's particles and their neighbours then share cache lines. A walk over a bucket
// visits the same particles in the same order in both orders, so every sum of every sweep is unchanged;
// the state (positions, velocities) is written back in sorted order, so the next step's sort, and every
// exported field, are the reference's.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace pcisph {

// Per bucket: cells_d[key] = its range in sorted order (the reference's table, reorder semantics);
// codes[key] = Morton code (8 bits per axis, 24 bits) of its first particle's cell, all ones when empty (the
// caller fills codes with 0xFF bytes first). Out-of-range sorted entries set status bit 4.
void launch_bucket_codes(const uint32_t* sorted_keys, const uint32_t* sorted_ids, const float4* state_pos,
                         uint32_t n, const DevParams& P, uint2* cells_d, uint32_t* codes, Control* ctl,
                         cudaStream_t s);

// Elements of scan scratch for bk buckets.
size_t working_ranges_scratch(uint32_t bk);
// order = bucket ids sorted by code; lengths from cells_d; cells_w[b] = range of bucket b in working order
// (exclusive scan of the lengths in `order`, clamped to [0, n]). Three launches.
void launch_working_ranges(const uint32_t* order, uint32_t bk, const uint2* cells_d, uint2* cells_w,
                           uint32_t* scratch, uint32_t n, cudaStream_t s);

// pos_w/vel_w[w] = state[sorted_ids[d]] for sorted index d at working index w; d_of_w and w_of_d.
void launch_permute(const uint32_t* sorted_keys, const uint32_t* sorted_ids, const float4* state_pos,
                    const float4* state_vel, uint32_t n, uint32_t bk, const uint2* cells_d, const uint2* cells_w,
                    float4* pos_w, float4* vel_w, uint32_t* d_of_w, uint32_t* w_of_d, Control* ctl, cudaStream_t s,
                    const float* state_skin = nullptr);

// dst[i] = src[idx[i]] and dst[idx[i]] = src[i] for float4 and float elements; iota: a[i] = i.
void launch_gather4(const float4* src, const uint32_t* idx, float4* dst, uint32_t n, cudaStream_t s);
void launch_gather1(const float* src, const uint32_t* idx, float* dst, uint32_t n, cudaStream_t s);
void launch_scatter4(const float4* src, const uint32_t* idx, float4* dst, uint32_t n, cudaStream_t s);
void launch_scatter1(const float* src, const uint32_t* idx, float* dst, uint32_t n, cudaStream_t s);
// out = (in.xyz, 0) (in place when out == in): the step's positions without the per-particle skin in w.
void launch_xyz0(const float4* in, float4* out, uint32_t n, cudaStream_t s);
void launch_iota(uint32_t* a, uint32_t n, cudaStream_t s);

}  // namespace pcisph
