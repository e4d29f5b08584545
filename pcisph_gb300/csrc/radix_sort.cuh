// radix_sort.cuh -- stable LSD radix sort of uint32 keys carrying uint32 values.
//
// Replaces clogs::Radixsort (libs/clogs/include/clogs/radixsort.h:176-191), whose
// contract is a stable key/value sort with an optional bound on key bits. Each
// digit pass is reduce-then-scan: per-tile digit counts (upsweep), a scan of
// every digit's tile counts (one CTA per digit), and a downsweep that ranks the
// tile's keys stably (warp match + per-warp counters, in element order), stages
// them in shared memory in digit order and writes each digit run coalesced.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace pcisph {

// Keys per tile of the sort kernels (256 threads x 16 keys).
constexpr size_t kRadixTile = 4096;

constexpr size_t radix_align256(size_t b) { return (b + 255) & ~size_t(255); }

// Scratch bytes of a sort of n elements with digit_bits-wide digits: alternate keys, alternate values,
// per-tile digit counts and digit totals, each 256-byte aligned.
constexpr size_t radix_scratch_bytes(size_t n, int digit_bits) {
    return 2 * radix_align256(n * sizeof(uint32_t)) +
           radix_align256(((size_t)1 << digit_bits) * ((n + kRadixTile - 1) / kRadixTile) * sizeof(uint32_t)) +
           radix_align256(((size_t)1 << digit_bits) * sizeof(uint32_t));
}

// Dynamic shared memory of the downsweep kernel for bits-wide digits (8 warps' 16-bit digit counters, two
// digit tables, the tile's keys and values). Above 48 KB the kernel needs radix_configure_kernels().
constexpr size_t radix_downsweep_smem(int bits) {
    return (size_t)8 * ((size_t)1 << bits) * sizeof(unsigned short) + 2 * ((size_t)1 << bits) * sizeof(uint32_t) +
           2 * kRadixTile * sizeof(uint32_t);
}

// Raise the dynamic shared-memory limit of the wide-digit kernels on the current device.
// Call once per device before the first sort (outside stream capture).
cudaError_t radix_configure_kernels();

struct RadixSortPlan {
    int digit_bits = 8;
    int passes = 0;
    size_t tiles = 0;
};

class RadixSorter {
   public:
    RadixSorter() = default;
    ~RadixSorter();
    RadixSorter(const RadixSorter&) = delete;
    RadixSorter& operator=(const RadixSorter&) = delete;

    // Scratch bytes needed for n elements (alternate keys/values + tile counts).
    static constexpr size_t scratch_bytes(size_t n, int digit_bits) { return radix_scratch_bytes(n, digit_bits); }
    // Use caller-provided scratch (must hold scratch_bytes); otherwise the sorter allocates lazily.
    void set_scratch(void* ptr, size_t bytes);
    void set_digit_bits(int bits) { digit_bits_ = bits; }
    int digit_bits() const { return digit_bits_; }

    // Sorts keys/values in place (result copied back if the pass count is odd, unless out_* are given).
    // If values_in_identity, the input values are taken as 0..n-1 and `values` is write-only.
    // Returns a cudaError_t. When out_keys/out_values are not null and the pass count is odd, the
    // result is left in the scratch buffers and *out_keys/*out_values point to it.
    cudaError_t sort(uint32_t* keys, uint32_t* values, size_t n, int bits, bool values_in_identity,
                     cudaStream_t stream, uint32_t** out_keys = nullptr, uint32_t** out_values = nullptr);
    // Kernel launches issued by the last sort() call.
    int last_launches() const { return last_launches_; }

   private:
    void* scratch_ = nullptr;
    size_t scratch_cap_ = 0;
    bool owns_ = false;
    int digit_bits_ = 8;
    int last_launches_ = 0;
};

}  // namespace pcisph
