// The stand-alone pair sort without any device allocation.
//
// Some callers cannot hand the sort a temporary buffer or let it allocate:
// code whose device memory is owned by another allocator (a framework's
// caching allocator that must stay the only one), frame loops with a fixed,
// preallocated memory budget where an allocation would stall the frame, and
// embedding hosts that forbid cudaMalloc after start-up. For them this file
// keeps the sort's scratch in a file-scope device array, sized for at most
// kNoAllocMaxLength pairs. Every GPU that loads the library holds the array
// (about 16 MiB) until the process exits.
//
// The array is shared by every call on a device and keeps what the last call
// left in it; the sort clears the parts that must start at zero (histograms,
// tile tickets, look-back words) at the start of each call. Calls that
// overlap on the GPU (for example on two streams) race on the array and
// corrupt each other's results; serialise them.
//
// The first call on a device resolves the array's device address there (with
// that device current) and caches it; make that first call before any stream
// capture begins.
#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace {

constexpr uint32_t kNoAllocMaxLength = ASTRO_RADIX_SORT_NOALLOC_MAX_LENGTH;

// Bytes of sort_plan(kNoAllocMaxLength, 64): the counters (error word
// included), 8 passes of 256-bin histograms, 8 passes of 256 look-back
// words per tile, 8 passes of 256-bin offsets and the ping-pong keys (8 B)
// and values (4 B), each region 256-aligned.
constexpr size_t kTiles = (kNoAllocMaxLength + astro::kSortPlanTile - 1) / astro::kSortPlanTile;
constexpr size_t kNoAllocBytes = 8ull * kNoAllocMaxLength + 4ull * kNoAllocMaxLength +
                                 4ull * 8 * 256 + 4ull * 8 * 256 + 256 + 4ull * 8 * kTiles * 256;

static __device__ __align__(256) unsigned char g_sort_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// Device address of g_sort_scratch on the current device (set up once).
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace

namespace astro {
// The static scratch of this device and its size (for the test hook).
cudaError_t noalloc_scratch(void** ptr, size_t* bytes) {
    *bytes = kNoAllocBytes;
    return scratch_address(ptr);
}
}  // namespace astro

// No counterpart in the reference: astro_radix_sort with the scratch in a
// static device array instead of caller-supplied memory.
extern "C" int astro_radix_sort_noalloc(const uint64_t* d_input, const uint32_t* d_input_indices,
                                        uint64_t* d_output, uint32_t* d_output_indices,
                                        uint32_t estimated_length, const uint32_t* d_actual_count,
                                        uint32_t key_bits, void* stream) {
    if (estimated_length == 0) return ASTRO_OK;
    if (!d_input || !d_output || !d_output_indices || key_bits > 64)
        return ASTRO_ERR_INVALID_ARGUMENT;
    if ((const void*)d_input == (const void*)d_output ||
        (const void*)d_input_indices == (const void*)d_output_indices)
        return ASTRO_ERR_INVALID_ARGUMENT;
    if (estimated_length > kNoAllocMaxLength) return ASTRO_ERR_CAPACITY;
    const size_t need = astro::sort_plan(estimated_length, key_bits).total;
    if (need > kNoAllocBytes) return ASTRO_ERR_CAPACITY;
    void* scratch = nullptr;
    if (scratch_address(&scratch) != cudaSuccess) {
        (void)cudaGetLastError();
        return ASTRO_ERR_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = astro::sort_pairs(d_input, d_input_indices, d_output, d_output_indices,
                                      estimated_length, d_actual_count, key_bits, scratch,
                                      kNoAllocBytes, st, nullptr);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return ASTRO_ERR_CUDA;
    }
    // On the NULL stream the call waits and reports the sort's device status
    // (a look-back wait that gave up); otherwise the caller reads it with
    // astro_radix_sort_noalloc_status once the stream has reached this sort.
    return st == nullptr ? astro::sort_status(scratch, st) : ASTRO_OK;
}

// The device status of the last no-alloc sort on the current device: waits
// for `stream`, then reads and clears the error word in the static array.
extern "C" int astro_radix_sort_noalloc_status(void* stream) {
    void* scratch = nullptr;
    if (scratch_address(&scratch) != cudaSuccess) {
        (void)cudaGetLastError();
        return ASTRO_ERR_CUDA;
    }
    return astro::sort_status(scratch, static_cast<cudaStream_t>(stream));
}
