// akua_sort_pairs_noalloc: the step's stable radix sort of (key, value) pairs for callers that
// cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc: host applications whose device memory is
// owned by their own allocator or held to a fixed budget (a game engine's or renderer's heap), and
// real-time frame loops where an allocation's implicit device synchronisation would stall the
// frame.  This entry point therefore keeps all of its temporary storage in one file-scope device
// array of fixed size; the caller passes only inputs and outputs.
//
// The array is shared by every call in the process, keeps the last call's contents, and is
// resident on every device that loads the library until the process exits.  Calls whose work
// overlaps on the GPU (different streams, or different host threads) race on it: the caller
// must order them.
#include <cstdint>
#include <cuda_runtime.h>
#include <mutex>

#include "akua_pbf.h"

// The sort kernels get internal linkage here so this translation unit can be linked next to the
// solver's, which instantiates the same header.
namespace {
#include "radix_sort.cuh"
}  // namespace

namespace {

constexpr int kMaxPairs = AKUA_SORT_NOALLOC_MAX_PAIRS;
constexpr size_t kTiles = ((size_t)kMaxPairs + akua::radix::TILE - 1) / akua::radix::TILE;
// one ping-pong buffer of keys and values, the (digit, tile) count matrix, per-pass digit totals
constexpr size_t kCountWords =
    (size_t)akua::radix::MAX_RADIX * kTiles + (size_t)akua::radix::MAX_PASSES * akua::radix::MAX_RADIX;
constexpr size_t kScratchWords = 2 * (size_t)kMaxPairs + kCountWords;

struct NoMark {
    void operator()(const char*) {}
};

// True when the byte ranges [a, a + bytes) and [b, b + bytes) share a byte.
bool overlap(const void* a, const void* b, size_t bytes) {
    if (!a || !b) return false;
    const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    return x < y + bytes && y < x + bytes;
}

}  // namespace

static __device__ __align__(256) uint32_t g_sort_scratch[kScratchWords];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
uint32_t* g_scratch[kMaxDevices] = {};

// Device address of g_sort_scratch on the current device, looked up on the first call per device
// and kept for the life of the process (a cudaDeviceReset between calls is not supported: it
// unloads the module that holds the array).  In host code the array's name is only a host-side
// stand-in; the kernels need this address.
cudaError_t scratch_address(uint32_t** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess) return e;
        g_scratch[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_scratch[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" int akua_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in,
                                       uint32_t* keys_out, uint32_t* vals_out, int32_t n,
                                       int32_t key_bits, void* stream) {
    if (n < 0 || key_bits < 1 || key_bits > 32) return AKUA_ERR_INVALID_ARGUMENT;
    if (n > kMaxPairs) return AKUA_ERR_TOO_LARGE;
    if (n == 0) return AKUA_OK;
    if (!keys_in || !keys_out || !vals_out) return AKUA_ERR_INVALID_ARGUMENT;
    // the passes read the inputs while other blocks write the outputs: no two of the four arrays
    // may share memory, except the two inputs (both are only read)
    const size_t bytes = sizeof(uint32_t) * (size_t)n;
    if (overlap(keys_out, vals_out, bytes) || overlap(keys_in, keys_out, bytes) ||
        overlap(keys_in, vals_out, bytes) || overlap(vals_in, keys_out, bytes) ||
        overlap(vals_in, vals_out, bytes))
        return AKUA_ERR_INVALID_ARGUMENT;
    uint32_t* scratch = nullptr;
    cudaError_t e = scratch_address(&scratch);
    if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? AKUA_ERR_OUT_OF_MEMORY : AKUA_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* tmp_keys = scratch;
    uint32_t* tmp_vals = scratch + kMaxPairs;
    uint32_t* counts = scratch + 2 * (size_t)kMaxPairs;
    uint32_t* totals = counts + (size_t)akua::radix::MAX_RADIX * akua::radix::num_tiles(n);
    // the digit totals accumulate atomically and must start at zero on every call
    e = cudaMemsetAsync(totals, 0,
                        sizeof(uint32_t) * akua::radix::MAX_PASSES * akua::radix::MAX_RADIX, st);
    if (e != cudaSuccess) return AKUA_ERR_CUDA;
    const akua::radix::Plan plan = akua::radix::make_plan(key_bits);
    NoMark mark;
    // pass p writes to the caller's output when (passes - 1 - p) is even, so the last pass does
    const uint32_t* kin = keys_in;
    const uint32_t* vin = vals_in;  // null: the payload is each key's index
    for (int p = 0; p < plan.passes; ++p) {
        const bool to_out = ((plan.passes - 1 - p) & 1) == 0;
        uint32_t* kout = to_out ? keys_out : tmp_keys;
        uint32_t* vout = to_out ? vals_out : tmp_vals;
        uint32_t* tot = totals + (size_t)p * akua::radix::MAX_RADIX;
        // the digit covers only this pass's bits, so key bits at and above key_bits never
        // influence the order (a pass narrower than 8 bits still runs the 8-bit kernels)
        const uint32_t mask = (1u << plan.width[p]) - 1u;
        if (plan.width[p] <= 8)
            akua::radix::run_pass<8>(st, kin, vin, kout, vout, counts, tot, n, plan.shift[p],
                                      nullptr, mark, mask);
        else if (plan.width[p] == 9)
            akua::radix::run_pass<9>(st, kin, vin, kout, vout, counts, tot, n, plan.shift[p],
                                      nullptr, mark, mask);
        else
            akua::radix::run_pass<10>(st, kin, vin, kout, vout, counts, tot, n, plan.shift[p],
                                      nullptr, mark, mask);
        kin = kout;
        vin = vout;
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? AKUA_OK : AKUA_ERR_CUDA;
}
