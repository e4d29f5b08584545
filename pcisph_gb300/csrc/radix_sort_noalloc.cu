// radix_sort_noalloc.cu -- a radix-sort entry point that allocates no device memory.
//
// pcisph_radixsort_enqueue() gets its scratch (the alternate key/value buffers and the per-tile digit
// counts) from cudaMalloc. Some callers cannot allow that at the point where they sort: a host
// component whose device memory is all handed out up front by a pool allocator (a cudaMalloc there can
// fail, or break the pool's accounting), a real-time loop in which an allocation would implicitly
// synchronise the device and stall other streams. pcisph_radixsort_enqueue_noalloc() serves them: its
// scratch is a file-scope __device__ array that is part of this library's GPU image. It is created when
// the library's GPU code is loaded on a device and stays reserved on every device that loads it until
// the process exits, so it is sized for a modest maximum of PCISPH_NOALLOC_SORT_MAX_ELEMENTS keys
// (1,048,576 keys: about 8.3 MB per device).
//
// Host code cannot use the array's name as a device address (on the host it names a stand-in), so every
// call looks the device address up with cudaGetSymbolAddress on the current device. The lookup allocates
// nothing and is cheap; it is not cached, because the address belongs to the CUDA context, and a context
// torn down and created again (cudaDeviceReset) may load the module at another address. The first call on
// a device may be the one that loads this library's GPU code there; make that first call before any
// stream capture.
#include <cuda_runtime.h>

#include <string>

#include "../../include/pcisph_gpu.h"
#include "radix_sort.cuh"

namespace pcisph {
int report_error(int code, const std::string& msg);  // context.cu: sets pcisph_last_error()
}

namespace {

constexpr size_t kMaxElements = PCISPH_NOALLOC_SORT_MAX_ELEMENTS;
constexpr int kDigitBits = 8;
// alternate keys + alternate values + per-tile digit counts + digit totals, as RadixSorter lays them out
constexpr size_t kScratchBytes = pcisph::RadixSorter::scratch_bytes(kMaxElements, kDigitBits);
static_assert(kScratchBytes == pcisph::radix_scratch_bytes(kMaxElements, kDigitBits), "scratch layout");
// this path never raises the kernels' shared-memory limit: the 8-bit downsweep must fit the default 48 KB
static_assert(pcisph::radix_downsweep_smem(kDigitBits) <= 48 * 1024, "8-bit downsweep exceeds 48 KB");

static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

// Device address of g_sort_scratch in the current device's context.
int scratch_for_current_device(void** out) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || !p)
        return pcisph::report_error(PCISPH_ERR_CUDA, std::string("cudaGetSymbolAddress of the sort scratch: ") +
                                                         cudaGetErrorString(e));
    *out = p;
    return PCISPH_OK;
}

}  // namespace

extern "C" int pcisph_radixsort_enqueue_noalloc(uint32_t* keys, uint32_t* values, size_t elements,
                                                unsigned int max_bits, void* stream) {
    if (elements > kMaxElements)
        return pcisph::report_error(PCISPH_ERR_INVALID_ARG,
                                    "pcisph_radixsort_enqueue_noalloc: " + std::to_string(elements) +
                                        " elements exceed its fixed scratch of " + std::to_string(kMaxElements) +
                                        " (use pcisph_radixsort_enqueue for larger sorts)");
    if (elements && (!keys || !values)) return pcisph::report_error(PCISPH_ERR_INVALID_ARG, "keys/values are NULL");
    if (max_bits > 32) return pcisph::report_error(PCISPH_ERR_INVALID_ARG, "max_bits > 32");
    if (elements == 0) return PCISPH_OK;
    void* scratch = nullptr;
    int rc = scratch_for_current_device(&scratch);
    if (rc != PCISPH_OK) return rc;
    // Every byte of the scratch that a pass reads is written earlier in the same pass (digit counts by the
    // upsweep, their scan and totals by the scan, keys and values by the downsweep), so nothing left by an
    // earlier call needs clearing. Calls that overlap on the GPU (different streams) share this one array
    // and race; order them on one stream or with events.
    pcisph::RadixSorter sorter;
    sorter.set_digit_bits(kDigitBits);
    sorter.set_scratch(scratch, kScratchBytes);
    cudaError_t e = sorter.sort(keys, values, elements, max_bits == 0 ? 32 : (int)max_bits, false,
                                static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return pcisph::report_error(PCISPH_ERR_CUDA, std::string("radix sort: ") + cudaGetErrorString(e));
    return PCISPH_OK;
}
