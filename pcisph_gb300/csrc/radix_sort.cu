// radix_sort.cu -- stable LSD radix sort (see radix_sort.cuh).
#include "radix_sort.cuh"

#include <algorithm>

namespace pcisph {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // 4096 keys per tile
static_assert(kTile == kRadixTile, "tile size shared with the scratch layout (radix_sort.cuh)");

constexpr size_t align256(size_t b) { return radix_align256(b); }

// Exclusive scan in place over s[0..count) in shared memory; returns the total. All threads call.
__device__ uint32_t block_exclusive_scan(uint32_t* s, int count, uint32_t* warp_tmp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int per = (count + kThreads - 1) / kThreads;
    const int beg = min(count, (int)threadIdx.x * per), end = min(count, beg + per);
    uint32_t sum = 0;
    for (int i = beg; i < end; ++i) sum += s[i];
    uint32_t x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tmp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kWarps ? warp_tmp[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kWarps) warp_tmp[lane] = w;
    }
    __syncthreads();
    uint32_t run = x - sum + (warp > 0 ? warp_tmp[warp - 1] : 0u);
    const uint32_t total = warp_tmp[kWarps - 1];
    for (int i = beg; i < end; ++i) {
        uint32_t v = s[i];
        s[i] = run;
        run += v;
    }
    __syncthreads();
    return total;
}

// Per-tile digit counts, counts laid out digit-major: counts[d * tiles + tile].
template <int BITS>
__global__ void __launch_bounds__(kThreads) k_upsweep(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                      uint32_t* __restrict__ counts, uint32_t tiles) {
    constexpr int RADIX = 1 << BITS;
    __shared__ uint32_t hist[RADIX];
    for (int d = threadIdx.x; d < RADIX; d += kThreads) hist[d] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kTile;
    const int lane = threadIdx.x & 31;
#pragma unroll 4
    for (int i = threadIdx.x; i < kTile; i += kThreads) {
        const size_t idx = base + i;
        const bool valid = idx < n;
        const uint32_t d = valid ? (__ldg(&keys[idx]) >> shift) & (RADIX - 1) : 0xFFFFFFFFu;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        if (valid && (peers & ((1u << lane) - 1u)) == 0u) atomicAdd(&hist[d], (uint32_t)__popc(peers));
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += kThreads) counts[(size_t)d * tiles + blockIdx.x] = hist[d];
}

// One block per digit: exclusive scan of that digit's tile counts; the row total goes to totals[d].
__global__ void __launch_bounds__(kThreads) k_scan_rows(uint32_t* __restrict__ counts, uint32_t tiles,
                                                        uint32_t* __restrict__ totals) {
    __shared__ uint32_t buf[kThreads * 4];
    __shared__ uint32_t warp_tmp[kWarps];
    uint32_t* row = counts + (size_t)blockIdx.x * tiles;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < tiles; base += kThreads * 4) {
        const int cnt = (int)min((uint32_t)(kThreads * 4), tiles - base);
        for (int i = threadIdx.x; i < kThreads * 4; i += kThreads) buf[i] = i < cnt ? row[base + i] : 0u;
        __syncthreads();
        const uint32_t total = block_exclusive_scan(buf, kThreads * 4, warp_tmp);
        for (int i = threadIdx.x; i < cnt; i += kThreads) row[base + i] = buf[i] + carry;
        carry += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) totals[blockIdx.x] = carry;
}

template <int BITS>
constexpr size_t downsweep_smem() {
    static_assert(kWarps == 8, "radix_downsweep_smem counts 8 warps");
    return radix_downsweep_smem(BITS);
}

// Stable rank within the tile, stage in digit order, write each digit run contiguously.
template <int BITS>
__global__ void __launch_bounds__(kThreads) k_downsweep(const uint32_t* __restrict__ keys_in,
                                                        const uint32_t* __restrict__ vals_in,
                                                        uint32_t* __restrict__ keys_out,
                                                        uint32_t* __restrict__ vals_out, uint32_t n, int shift,
                                                        const uint32_t* __restrict__ tile_offsets,
                                                        const uint32_t* __restrict__ totals, uint32_t tiles) {
    constexpr int RADIX = 1 << BITS;
    constexpr uint32_t MASK = RADIX - 1;
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned short* whist = reinterpret_cast<unsigned short*>(smem);              // [kWarps][RADIX]
    uint32_t* local_start = reinterpret_cast<uint32_t*>(whist + kWarps * RADIX);  // [RADIX]
    uint32_t* gofs = local_start + RADIX;                                         // [RADIX]
    uint32_t* skeys = gofs + RADIX;                                               // [kTile]
    uint32_t* svals = skeys + kTile;                                              // [kTile]
    __shared__ uint32_t warp_tmp[kWarps];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t tile_base = (size_t)blockIdx.x * kTile;
    const uint32_t tile_n = (uint32_t)min((size_t)kTile, (size_t)n - tile_base);
    for (int i = threadIdx.x; i < kWarps * RADIX; i += kThreads) whist[i] = 0;
    __syncthreads();

    uint32_t k[kItems], v[kItems];
    unsigned short rk[kItems];
    const size_t wbase = tile_base + (size_t)warp * 32 * kItems;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const size_t idx = wbase + it * 32 + lane;
        const bool valid = idx < n;
        k[it] = valid ? __ldg(&keys_in[idx]) : 0u;
        v[it] = valid ? (vals_in ? __ldg(&vals_in[idx]) : (uint32_t)idx) : 0u;
    }
    unsigned short* my_hist = whist + warp * RADIX;
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        const bool valid = wbase + it * 32 + lane < n;
        const uint32_t d = valid ? (k[it] >> shift) & MASK : 0xFFFFFFFFu;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned lower = peers & ((1u << lane) - 1u);
        const unsigned short cur = valid ? my_hist[d] : (unsigned short)0;
        rk[it] = (unsigned short)(cur + __popc(lower));
        __syncwarp();
        if (valid && lower == 0u) my_hist[d] = (unsigned short)(cur + __popc(peers));
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += kThreads) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = whist[w * RADIX + d];
            whist[w * RADIX + d] = (unsigned short)run;
            run += c;
        }
        local_start[d] = run;
        gofs[d] = totals[d];
    }
    __syncthreads();
    block_exclusive_scan(local_start, RADIX, warp_tmp);
    block_exclusive_scan(gofs, RADIX, warp_tmp);
    for (int d = threadIdx.x; d < RADIX; d += kThreads) gofs[d] += tile_offsets[(size_t)d * tiles + blockIdx.x];
    __syncthreads();
#pragma unroll
    for (int it = 0; it < kItems; ++it) {
        if (wbase + it * 32 + lane < n) {
            const uint32_t d = (k[it] >> shift) & MASK;
            const uint32_t pos = local_start[d] + my_hist[d] + rk[it];
            skeys[pos] = k[it];
            svals[pos] = v[it];
        }
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < tile_n; i += kThreads) {
        const uint32_t key = skeys[i];
        const uint32_t d = (key >> shift) & MASK;
        const uint32_t o = gofs[d] + (i - local_start[d]);
        keys_out[o] = key;
        vals_out[o] = svals[i];
    }
}

template <int BITS>
cudaError_t run_pass(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout, uint32_t n,
                     int shift, uint32_t* counts, uint32_t* totals, uint32_t tiles, cudaStream_t s) {
    constexpr size_t smem = downsweep_smem<BITS>();
    k_upsweep<BITS><<<tiles, kThreads, 0, s>>>(kin, n, shift, counts, tiles);
    k_scan_rows<<<1 << BITS, kThreads, 0, s>>>(counts, tiles, totals);
    k_downsweep<BITS><<<tiles, kThreads, smem, s>>>(kin, vin, kout, vout, n, shift, counts, totals, tiles);
    return cudaGetLastError();
}

cudaError_t dispatch_pass(int bits, const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                          uint32_t n, int shift, uint32_t* counts, uint32_t* totals, uint32_t tiles,
                          cudaStream_t s) {
    switch (bits) {
        case 4: return run_pass<4>(kin, vin, kout, vout, n, shift, counts, totals, tiles, s);
        case 5: return run_pass<5>(kin, vin, kout, vout, n, shift, counts, totals, tiles, s);
        case 6: return run_pass<6>(kin, vin, kout, vout, n, shift, counts, totals, tiles, s);
        case 7: return run_pass<7>(kin, vin, kout, vout, n, shift, counts, totals, tiles, s);
        case 8: return run_pass<8>(kin, vin, kout, vout, n, shift, counts, totals, tiles, s);
        case 9: return run_pass<9>(kin, vin, kout, vout, n, shift, counts, totals, tiles, s);
        case 10: return run_pass<10>(kin, vin, kout, vout, n, shift, counts, totals, tiles, s);
        case 11: return run_pass<11>(kin, vin, kout, vout, n, shift, counts, totals, tiles, s);
        default: return cudaErrorInvalidValue;
    }
}

template <int BITS>
cudaError_t configure_one() {
    constexpr size_t smem = downsweep_smem<BITS>();
    if (smem <= 48 * 1024) return cudaSuccess;
    return cudaFuncSetAttribute(k_downsweep<BITS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

}  // namespace

cudaError_t radix_configure_kernels() {
    cudaError_t e = cudaSuccess;
    for (cudaError_t r : {configure_one<4>(), configure_one<5>(), configure_one<6>(), configure_one<7>(),
                          configure_one<8>(), configure_one<9>(), configure_one<10>(), configure_one<11>()})
        if (r != cudaSuccess) e = r;
    return e;
}

RadixSorter::~RadixSorter() {
    if (owns_ && scratch_) cudaFree(scratch_);
}

void RadixSorter::set_scratch(void* ptr, size_t bytes) {
    if (owns_ && scratch_) cudaFree(scratch_);
    scratch_ = ptr;
    scratch_cap_ = bytes;
    owns_ = false;
}

cudaError_t RadixSorter::sort(uint32_t* keys, uint32_t* values, size_t n, int bits, bool values_in_identity,
                              cudaStream_t stream, uint32_t** out_keys, uint32_t** out_values) {
    last_launches_ = 0;
    if (out_keys) *out_keys = keys;
    if (out_values) *out_values = values;
    if (n == 0) return cudaSuccess;
    if (n > 0xFFFFFFFFull) return cudaErrorInvalidValue;
    if (bits <= 0 || bits > 32) bits = 32;
    const int db = digit_bits_;
    if (db < 4 || db > 11) return cudaErrorInvalidValue;
    const size_t need = scratch_bytes(n, db);
    if (scratch_cap_ < need) {
        if (!owns_ && scratch_) return cudaErrorInvalidValue;  // caller scratch too small
        if (scratch_) cudaFree(scratch_);
        scratch_ = nullptr;
        scratch_cap_ = 0;
        cudaError_t e = cudaMalloc(&scratch_, need);
        if (e != cudaSuccess) return e;
        scratch_cap_ = need;
        owns_ = true;
    }
    const uint32_t tiles = (uint32_t)((n + kTile - 1) / kTile);
    unsigned char* p = static_cast<unsigned char*>(scratch_);
    uint32_t* alt_k = reinterpret_cast<uint32_t*>(p);
    p += align256(n * sizeof(uint32_t));
    uint32_t* alt_v = reinterpret_cast<uint32_t*>(p);
    p += align256(n * sizeof(uint32_t));
    uint32_t* counts = reinterpret_cast<uint32_t*>(p);
    p += align256(((size_t)1 << db) * tiles * sizeof(uint32_t));
    uint32_t* totals = reinterpret_cast<uint32_t*>(p);

    const int passes = (bits + db - 1) / db;
    uint32_t *sk = keys, *sv = values, *dk = alt_k, *dv = alt_v;
    for (int pass = 0; pass < passes; ++pass) {
        const uint32_t* vin = (pass == 0 && values_in_identity) ? nullptr : sv;
        cudaError_t e = dispatch_pass(db, sk, vin, dk, dv, (uint32_t)n, pass * db, counts, totals, tiles, stream);
        if (e != cudaSuccess) return e;
        last_launches_ += 3;
        std::swap(sk, dk);
        std::swap(sv, dv);
    }
    if (sk != keys) {
        if (out_keys && out_values) {
            *out_keys = sk;
            *out_values = sv;
        } else {
            cudaError_t e = cudaMemcpyAsync(keys, sk, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(values, sv, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, stream);
            if (e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

}  // namespace pcisph
