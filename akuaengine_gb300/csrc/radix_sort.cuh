// Stable LSD radix sort of (u32 key, u32 value) pairs.
//
// Replaces the comparison sort of whole 108-byte particle records in the reference
// (thrust::sort with a.hash < b.hash, NeighbourSearchCUDA.cu:167-170).  Only the keys and a u32
// payload move; the particle state is gathered once afterwards.  Stability makes ties keep the
// incoming order, i.e. the previous step's sorted order, which is what the reference's merge sort
// yields for equal hashes.
//
// Each pass handles RADIX_BITS bits with three kernels: per-tile digit counts, one exclusive scan
// over the (digit, tile) matrix, and a stable scatter in which warps rank their keys with
// match.any and per-warp running digit counters in shared memory.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace akua {
namespace radix {

constexpr int RADIX_BITS = 8;
constexpr int RADIX = 1 << RADIX_BITS;
constexpr int BLOCK = 256;
constexpr int WARPS = BLOCK / 32;
constexpr int ROUNDS = 16;                 // keys per lane
constexpr int WARP_ITEMS = ROUNDS * 32;    // 512
constexpr int TILE = WARPS * WARP_ITEMS;   // 4096 keys per tile
constexpr int SCAN_BLOCK = 1024;

inline int num_tiles(int n) { return (n + TILE - 1) / TILE; }

// counts[digit * tiles + tile] = number of keys of `tile` whose digit at `shift` is `digit`.
__global__ void __launch_bounds__(BLOCK) upsweep(const uint32_t* __restrict__ keys, int n, int shift,
                                                 uint32_t* __restrict__ counts, int tiles) {
    __shared__ uint32_t hist[WARPS][RADIX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = threadIdx.x; t < WARPS * RADIX; t += BLOCK) (&hist[0][0])[t] = 0;
    __syncthreads();
    const int base = blockIdx.x * TILE + warp * WARP_ITEMS + lane;
#pragma unroll 4
    for (int r = 0; r < ROUNDS; ++r) {
        const int idx = base + r * 32;
        if (idx < n) {
            const uint32_t d = (keys[idx] >> shift) & (RADIX - 1);
            atomicAdd(&hist[warp][d], 1u);
        }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += BLOCK) {
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) s += hist[w][d];
        counts[(size_t)d * tiles + blockIdx.x] = s;
    }
}

// In-place exclusive scan of `len` counts by one block.
__global__ void __launch_bounds__(SCAN_BLOCK) scan(uint32_t* __restrict__ counts, int len) {
    __shared__ uint32_t warp_sums[SCAN_BLOCK / 32];
    __shared__ uint32_t carry_s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry_s = 0;
    __syncthreads();
    constexpr int PER = 4;
    for (int chunk = 0; chunk < len; chunk += SCAN_BLOCK * PER) {
        const int i0 = chunk + threadIdx.x * PER;
        uint32_t v[PER];
        uint32_t local = 0;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            v[k] = (i0 + k < len) ? counts[i0 + k] : 0u;
            local += v[k];
        }
        // inclusive warp scan of per-thread sums
        uint32_t incl = local;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) warp_sums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t ws = warp_sums[lane];
            uint32_t wincl = ws;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, wincl, o);
                if (lane >= o) wincl += y;
            }
            warp_sums[lane] = wincl - ws;  // exclusive
        }
        __syncthreads();
        const uint32_t carry = carry_s;
        uint32_t run = carry + warp_sums[warp] + (incl - local);
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            if (i0 + k < len) counts[i0 + k] = run;
            run += v[k];
        }
        __syncthreads();
        if (threadIdx.x == SCAN_BLOCK - 1) carry_s = run;
        __syncthreads();
    }
}

// Stable scatter of one tile.  `vals_in == nullptr` means the payload is the key's index.
__global__ void __launch_bounds__(BLOCK)
    downsweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
              uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int n, int shift,
              const uint32_t* __restrict__ offsets, int tiles) {
    __shared__ uint32_t wbase[WARPS][RADIX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = threadIdx.x; t < WARPS * RADIX; t += BLOCK) (&wbase[0][0])[t] = 0;
    __syncthreads();
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int base = blockIdx.x * TILE + warp * WARP_ITEMS + lane;
    uint32_t key[ROUNDS], val[ROUNDS];
    uint16_t rank[ROUNDS];
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const int idx = base + r * 32;
        const bool valid = idx < n;
        key[r] = valid ? keys_in[idx] : 0xffffffffu;
        val[r] = valid ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0u;
        const uint32_t d = valid ? ((key[r] >> shift) & (RADIX - 1)) : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = 0;
        if (valid) before = wbase[warp][d];
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wbase[warp][d] = before + __popc(peers);
        __syncwarp();
        rank[r] = (uint16_t)(before + __popc(peers & lt_mask));
    }
    __syncthreads();
    // exclusive prefix over warps per digit, plus the tile's global offset
    for (int d = threadIdx.x; d < RADIX; d += BLOCK) {
        uint32_t run = offsets[(size_t)d * tiles + blockIdx.x];
#pragma unroll
        for (int w = 0; w < WARPS; ++w) {
            const uint32_t c = wbase[w][d];
            wbase[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const int idx = base + r * 32;
        if (idx < n) {
            const uint32_t d = (key[r] >> shift) & (RADIX - 1);
            const uint32_t dst = wbase[warp][d] + rank[r];
            keys_out[dst] = key[r];
            vals_out[dst] = val[r];
        }
    }
}

// Number of passes for keys below `bound` (bound >= 1).
inline int passes_for(uint32_t bound) {
    int bits = 0;
    uint64_t b = (uint64_t)bound - 1;
    while (b) { ++bits; b >>= 1; }
    if (bits == 0) bits = 1;
    return (bits + RADIX_BITS - 1) / RADIX_BITS;
}

// Sorts keys[0..n) with payload (index on input).  Ping-pongs between (k0, v0) and (k1, v1);
// returns true if the result ended in (k1, v1).  `counts` holds RADIX * num_tiles(n) words.
// `mark(name)` is called after every launch.
template <class Mark>
inline bool sort_pairs(cudaStream_t s, uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1,
                       uint32_t* counts, int n, int passes, Mark&& mark) {
    const int tiles = num_tiles(n);
    uint32_t *kin = k0, *vin = nullptr, *kout = k1, *vout = v1;
    for (int p = 0; p < passes; ++p) {
        const int shift = p * RADIX_BITS;
        upsweep<<<tiles, BLOCK, 0, s>>>(kin, n, shift, counts, tiles);
        mark("radix_upsweep");
        scan<<<1, SCAN_BLOCK, 0, s>>>(counts, RADIX * tiles);
        mark("radix_scan");
        downsweep<<<tiles, BLOCK, 0, s>>>(kin, vin, kout, vout, n, shift, counts, tiles);
        mark("radix_downsweep");
        // next pass reads what this one wrote
        uint32_t* nk = kout;
        uint32_t* nv = vout;
        kout = kin;
        vout = (vin ? vin : v0);
        kin = nk;
        vin = nv;
    }
    return kin == k1;
}

}  // namespace radix
}  // namespace akua
