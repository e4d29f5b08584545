// spatial_order.cu -- working order of a step: buckets placed in Morton order of their cells.
#include "spatial_order.cuh"

namespace pcisph {
namespace {

constexpr int kBlock = 256;
constexpr int kRounds = 16;                     // elements per thread in the range scan
constexpr int kScanTile = kBlock * kRounds;     // elements per block
inline unsigned grid_for(uint32_t n) { return (n + kBlock - 1) / kBlock; }

// 8 low bits of v spread to every third bit (bit k -> bit 3k)
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 0xFFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__global__ void __launch_bounds__(kBlock) k_bucket_codes(const uint32_t* __restrict__ sk, const uint32_t* __restrict__ sv,
                                                         const float4* __restrict__ state_pos, uint32_t n, DevParams P,
                                                         uint2* __restrict__ cells_d, uint32_t* __restrict__ codes,
                                                         Control* ctl) {
    const uint32_t d = blockIdx.x * kBlock + threadIdx.x;
    if (d >= n) return;
    const uint32_t key = sk[d], src = sv[d];
    if (key >= P.bucket_count || src >= n) {  // a sort that broke its contract: flag it, touch nothing
        atomicOr(&ctl->status, 4u);
        return;
    }
    if (d == 0 || key != sk[d - 1]) {
        cells_d[key].x = d;
        const float4 p = state_pos[src];
        const Cell c = cell_of(p.x, p.y, p.z, P);
        codes[key] = spread3(c.x) | (spread3(c.y) << 1) | (spread3(c.z) << 2);
    }
    if (d == n - 1 || key != sk[d + 1]) cells_d[key].y = d + 1;
}

__device__ __forceinline__ uint32_t range_len(const uint2* __restrict__ cells_d, const uint32_t* __restrict__ order,
                                              uint32_t q, uint32_t bk) {
    if (q >= bk) return 0u;
    const uint2 r = cells_d[order[q]];
    return r.y > r.x ? r.y - r.x : 0u;
}

// exclusive scan of v over the block; *total gets the block sum
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
    __shared__ uint32_t warp_tot[kBlock / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    uint32_t before = 0, sum = 0;
#pragma unroll
    for (int w = 0; w < kBlock / 32; ++w) {
        const uint32_t t = warp_tot[w];
        before += w < warp ? t : 0u;
        sum += t;
    }
    __syncthreads();  // warp_tot is reused by the next call
    *total = sum;
    return before + x - v;
}

__global__ void __launch_bounds__(kBlock) k_range_tile_sums(const uint32_t* __restrict__ order, uint32_t bk,
                                                            const uint2* __restrict__ cells_d,
                                                            uint32_t* __restrict__ sums) {
    const uint32_t base = blockIdx.x * kScanTile;
    uint32_t acc = 0;
#pragma unroll 4
    for (int r = 0; r < kRounds; ++r) acc += range_len(cells_d, order, base + r * kBlock + threadIdx.x, bk);
    acc = __reduce_add_sync(0xffffffffu, acc);
    __shared__ uint32_t part[kBlock / 32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
#pragma unroll
        for (int w = 0; w < kBlock / 32; ++w) t += part[w];
        sums[blockIdx.x] = t;
    }
}

// one block: exclusive scan of the tile sums in place
__global__ void __launch_bounds__(kBlock) k_range_scan_sums(uint32_t* sums, uint32_t tiles) {
    uint32_t carry = 0;
    for (uint32_t base = 0; base < tiles; base += kBlock) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < tiles ? sums[i] : 0u;
        uint32_t total;
        const uint32_t ex = block_exclusive_scan(v, &total);
        if (i < tiles) sums[i] = carry + ex;
        carry += total;
    }
}

// ranges are clamped to [0, n]: a sort that broke its contract (flagged) cannot send a sweep out of bounds
__global__ void __launch_bounds__(kBlock) k_range_write(const uint32_t* __restrict__ order, uint32_t bk,
                                                        const uint2* __restrict__ cells_d,
                                                        const uint32_t* __restrict__ sums, uint2* __restrict__ cells_w,
                                                        uint32_t n) {
    const uint32_t base = blockIdx.x * kScanTile;
    uint32_t carry = sums[blockIdx.x];
    for (int r = 0; r < kRounds; ++r) {
        const uint32_t q = base + r * kBlock + threadIdx.x;
        const uint32_t len = range_len(cells_d, order, q, bk);
        uint32_t total;
        const uint32_t ex = block_exclusive_scan(len, &total);
        if (q < bk) {
            const uint32_t start = min(carry + ex, n);
            cells_w[order[q]] = make_uint2(start, min(start + len, n));
        }
        carry += total;
    }
}

__global__ void __launch_bounds__(kBlock) k_permute(const uint32_t* __restrict__ sk, const uint32_t* __restrict__ sv,
                                                    const float4* __restrict__ state_pos,
                                                    const float4* __restrict__ state_vel, uint32_t n, uint32_t bk,
                                                    const uint2* __restrict__ cells_d, const uint2* __restrict__ cells_w,
                                                    float4* __restrict__ pos_w, float4* __restrict__ vel_w,
                                                    uint32_t* __restrict__ d_of_w, uint32_t* __restrict__ w_of_d,
                                                    Control* ctl, const float* __restrict__ state_skin) {
    const uint32_t d = blockIdx.x * kBlock + threadIdx.x;
    if (d >= n) return;
    const uint32_t key = sk[d], src = sv[d];
    if (key >= bk || src >= n) return;  // flagged by k_bucket_codes
    const uint2 rd = cells_d[key], rw = cells_w[key];
    const uint32_t w = rw.x + (d - rd.x);
    if (d < rd.x || w >= n) {
        atomicOr(&ctl->status, 4u);
        return;
    }
    float4 p = state_pos[src];
    if (state_skin) p.w = state_skin[src];  // the particle's stored half skin rides in w
    pos_w[w] = p;
    vel_w[w] = state_vel[src];
    d_of_w[w] = d;
    w_of_d[d] = w;
}

__global__ void __launch_bounds__(kBlock) k_gather4(const float4* __restrict__ src, const uint32_t* __restrict__ idx,
                                                    float4* __restrict__ dst, uint32_t n) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < n) {
        const uint32_t j = idx[i];
        if (j < n) dst[i] = src[j];
    }
}
__global__ void __launch_bounds__(kBlock) k_gather1(const float* __restrict__ src, const uint32_t* __restrict__ idx,
                                                    float* __restrict__ dst, uint32_t n) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < n) {
        const uint32_t j = idx[i];
        if (j < n) dst[i] = src[j];
    }
}
__global__ void __launch_bounds__(kBlock) k_scatter4(const float4* __restrict__ src, const uint32_t* __restrict__ idx,
                                                     float4* __restrict__ dst, uint32_t n) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < n) {
        const uint32_t j = idx[i];
        if (j < n) dst[j] = src[i];
    }
}
__global__ void __launch_bounds__(kBlock) k_scatter1(const float* __restrict__ src, const uint32_t* __restrict__ idx,
                                                     float* __restrict__ dst, uint32_t n) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < n) {
        const uint32_t j = idx[i];
        if (j < n) dst[j] = src[i];
    }
}
// out[i] = (in[i].xyz, 0); in place when out == in
__global__ void __launch_bounds__(kBlock) k_xyz0(const float4* in, float4* out, uint32_t n) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < n) {
        const float4 v = in[i];
        out[i] = make_float4(v.x, v.y, v.z, 0.f);
    }
}
__global__ void __launch_bounds__(kBlock) k_iota(uint32_t* a, uint32_t n) {
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i < n) a[i] = i;
}

}  // namespace

void launch_bucket_codes(const uint32_t* sorted_keys, const uint32_t* sorted_ids, const float4* state_pos,
                         uint32_t n, const DevParams& P, uint2* cells_d, uint32_t* codes, Control* ctl,
                         cudaStream_t s) {
    if (n) k_bucket_codes<<<grid_for(n), kBlock, 0, s>>>(sorted_keys, sorted_ids, state_pos, n, P, cells_d, codes, ctl);
}

size_t working_ranges_scratch(uint32_t bk) { return (bk + kScanTile - 1) / kScanTile + 1; }

void launch_working_ranges(const uint32_t* order, uint32_t bk, const uint2* cells_d, uint2* cells_w,
                           uint32_t* scratch, uint32_t n, cudaStream_t s) {
    const uint32_t tiles = (bk + kScanTile - 1) / kScanTile;
    if (!tiles) return;
    k_range_tile_sums<<<tiles, kBlock, 0, s>>>(order, bk, cells_d, scratch);
    k_range_scan_sums<<<1, kBlock, 0, s>>>(scratch, tiles);
    k_range_write<<<tiles, kBlock, 0, s>>>(order, bk, cells_d, scratch, cells_w, n);
}

void launch_permute(const uint32_t* sorted_keys, const uint32_t* sorted_ids, const float4* state_pos,
                    const float4* state_vel, uint32_t n, uint32_t bk, const uint2* cells_d, const uint2* cells_w,
                    float4* pos_w, float4* vel_w, uint32_t* d_of_w, uint32_t* w_of_d, Control* ctl, cudaStream_t s,
                    const float* state_skin) {
    if (n)
        k_permute<<<grid_for(n), kBlock, 0, s>>>(sorted_keys, sorted_ids, state_pos, state_vel, n, bk, cells_d, cells_w,
                                                 pos_w, vel_w, d_of_w, w_of_d, ctl, state_skin);
}

void launch_gather4(const float4* src, const uint32_t* idx, float4* dst, uint32_t n, cudaStream_t s) {
    if (n) k_gather4<<<grid_for(n), kBlock, 0, s>>>(src, idx, dst, n);
}
void launch_gather1(const float* src, const uint32_t* idx, float* dst, uint32_t n, cudaStream_t s) {
    if (n) k_gather1<<<grid_for(n), kBlock, 0, s>>>(src, idx, dst, n);
}
void launch_scatter4(const float4* src, const uint32_t* idx, float4* dst, uint32_t n, cudaStream_t s) {
    if (n) k_scatter4<<<grid_for(n), kBlock, 0, s>>>(src, idx, dst, n);
}
void launch_scatter1(const float* src, const uint32_t* idx, float* dst, uint32_t n, cudaStream_t s) {
    if (n) k_scatter1<<<grid_for(n), kBlock, 0, s>>>(src, idx, dst, n);
}
void launch_xyz0(const float4* in, float4* out, uint32_t n, cudaStream_t s) {
    if (n) k_xyz0<<<grid_for(n), kBlock, 0, s>>>(in, out, n);
}
void launch_iota(uint32_t* a, uint32_t n, cudaStream_t s) {
    if (n) k_iota<<<grid_for(n), kBlock, 0, s>>>(a, n);
}

}  // namespace pcisph
