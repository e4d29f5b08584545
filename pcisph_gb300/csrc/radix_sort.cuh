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
    static size_t scratch_bytes(size_t n, int digit_bits);
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
