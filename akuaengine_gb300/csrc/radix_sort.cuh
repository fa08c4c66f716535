// Stable LSD radix sort of (u32 key, u32 value) pairs.
//
// Replaces the comparison sort of whole 108-byte particle records in the reference
// (thrust::sort with a.hash < b.hash, NeighbourSearchCUDA.cu:167-170).  Only keys and a u32
// payload move; particle state is gathered once afterwards.  Stability makes equal keys keep their
// incoming order — for the cell-hash sort that is the previous step's sorted order, which is what
// the reference's merge sort yields for equal hashes.
//
// A sort of `bits`-bit keys runs ceil(bits / 10) passes of equal digit width (8..10 bits).  Each
// pass: per-tile digit counts (also accumulated into per-digit totals), one block per digit that
// turns its row of the (digit, tile) count matrix into global offsets, and a stable scatter in
// which warps rank their keys with match.any and per-warp running digit counters.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace akua {
namespace radix {

constexpr int MAX_BITS = 10;
constexpr int MAX_RADIX = 1 << MAX_BITS;
constexpr int BLOCK = 256;
constexpr int WARPS = BLOCK / 32;
constexpr int ROUNDS = 16;                // keys per lane
constexpr int WARP_ITEMS = ROUNDS * 32;   // 512
constexpr int TILE = WARPS * WARP_ITEMS;  // 4096 keys per tile
constexpr int SCAN_BLOCK = 256;
constexpr int MAX_PASSES = 4;

inline int num_tiles(int n) { return (n + TILE - 1) / TILE; }

// Digit width per pass for keys of `bits` significant bits.
struct Plan {
    int passes = 0;
    int width[MAX_PASSES] = {0, 0, 0, 0};
    int shift[MAX_PASSES] = {0, 0, 0, 0};
};

inline Plan make_plan(int bits) {
    Plan p;
    if (bits < 1) bits = 1;
    p.passes = (bits + MAX_BITS - 1) / MAX_BITS;
    int shift = 0, left = bits;
    for (int k = 0; k < p.passes; ++k) {
        const int w0 = (left + (p.passes - k) - 1) / (p.passes - k);
        const int w = w0 < 8 ? (left < 8 ? left : 8) : w0;  // widths below 8 gain nothing
        p.width[k] = w;
        p.shift[k] = shift;
        shift += w;
        left -= w;
        if (left <= 0) { p.passes = k + 1; break; }
    }
    return p;
}

inline int bits_for(uint64_t bound) {  // keys are < bound
    int bits = 0;
    uint64_t b = bound > 0 ? bound - 1 : 0;
    while (b) { ++bits; b >>= 1; }
    return bits < 1 ? 1 : bits;
}

// counts[d * tiles + tile] = keys of `tile` with digit d; totals[d] += the same.  A key's digit
// is (key >> shift) & digit_mask; digit_mask < RADIX narrows a pass to fewer bits than BITS.
template <int BITS>
__global__ void __launch_bounds__(BLOCK) upsweep(const uint32_t* __restrict__ keys, int n, int shift,
                                                 uint32_t digit_mask, uint32_t* __restrict__ counts,
                                                 uint32_t* __restrict__ totals, int tiles) {
    constexpr int RADIX = 1 << BITS;
    __shared__ uint32_t hist[WARPS][RADIX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = threadIdx.x; t < WARPS * RADIX; t += BLOCK) (&hist[0][0])[t] = 0;
    __syncthreads();
    const int base = blockIdx.x * TILE + warp * WARP_ITEMS + lane;
#pragma unroll 4
    for (int r = 0; r < ROUNDS; ++r) {
        const int idx = base + r * 32;
        if (idx < n) atomicAdd(&hist[warp][(keys[idx] >> shift) & digit_mask], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RADIX; d += BLOCK) {
        uint32_t s = 0;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) s += hist[w][d];
        counts[(size_t)d * tiles + blockIdx.x] = s;
        if (s) atomicAdd(&totals[d], s);
    }
}

// Block d: offsets[d][t] = sum of totals[0..d) + sum of counts[d][0..t).
__global__ void __launch_bounds__(SCAN_BLOCK) scan_rows(uint32_t* __restrict__ counts,
                                                        const uint32_t* __restrict__ totals,
                                                        int tiles) {
    __shared__ uint32_t red[SCAN_BLOCK / 32];
    __shared__ uint32_t carry_s;
    const int d = blockIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t part = 0;
    for (int k = threadIdx.x; k < d; k += SCAN_BLOCK) part += totals[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) red[warp] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t b = 0;
        for (int w = 0; w < SCAN_BLOCK / 32; ++w) b += red[w];
        carry_s = b;
    }
    __syncthreads();
    uint32_t* row = counts + (size_t)d * tiles;
    for (int chunk = 0; chunk < tiles; chunk += SCAN_BLOCK) {
        const int t = chunk + threadIdx.x;
        const uint32_t v = t < tiles ? row[t] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        __syncthreads();  // red[] reuse
        if (lane == 31) red[warp] = incl;
        __syncthreads();
        uint32_t wpre = 0;
        for (int w = 0; w < warp; ++w) wpre += red[w];
        const uint32_t carry = carry_s;
        if (t < tiles) row[t] = carry + wpre + incl - v;
        __syncthreads();
        if (threadIdx.x == SCAN_BLOCK - 1) carry_s = carry + wpre + incl;
        __syncthreads();
    }
}

// Stable scatter of one tile.  `vals_in == nullptr` means the payload is the key's index.  With
// `rank_out`, rank_out[payload] = the pair's output position too (the inverse permutation).
template <int BITS>
__global__ void __launch_bounds__(BLOCK)
    downsweep(const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
              uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int n, int shift,
              uint32_t digit_mask, const uint32_t* __restrict__ offsets, int tiles,
              uint32_t* __restrict__ rank_out) {
    constexpr int RADIX = 1 << BITS;
    extern __shared__ uint32_t wbase_flat[];  // [WARPS][RADIX]
    uint32_t(*wbase)[RADIX] = reinterpret_cast<uint32_t(*)[RADIX]>(wbase_flat);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int t = threadIdx.x; t < WARPS * RADIX; t += BLOCK) wbase_flat[t] = 0;
    __syncthreads();
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int base = blockIdx.x * TILE + warp * WARP_ITEMS + lane;
    uint32_t key[ROUNDS], val[ROUNDS];
    uint16_t rank[ROUNDS];
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const int idx = base + r * 32;
        const bool valid = idx < n;
        key[r] = valid ? keys_in[idx] : 0u;
        val[r] = valid ? (vals_in ? vals_in[idx] : (uint32_t)idx) : 0u;
    }
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const int idx = base + r * 32;
        const bool valid = idx < n;
        const uint32_t d = valid ? ((key[r] >> shift) & digit_mask) : 0xffffffffu;
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        uint32_t before = 0;
        if (valid) before = wbase[warp][d];
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wbase[warp][d] = before + __popc(peers);
        __syncwarp();
        rank[r] = (uint16_t)(before + __popc(peers & lt_mask));
    }
    __syncthreads();
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
            const uint32_t d = (key[r] >> shift) & digit_mask;
            const uint32_t dst = wbase[warp][d] + rank[r];
            keys_out[dst] = key[r];
            vals_out[dst] = val[r];
            if (rank_out) rank_out[val[r]] = dst;
        }
    }
}

// One pass over the digit (key >> shift) & digit_mask; digit_mask defaults to all BITS bits.
template <int BITS, class Mark>
inline void run_pass(cudaStream_t s, const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                     uint32_t* vout, uint32_t* counts, uint32_t* totals, int n, int shift,
                     uint32_t* rank_out, Mark& mark, uint32_t digit_mask = (1u << BITS) - 1u) {
    const int tiles = num_tiles(n);
    constexpr int RADIX = 1 << BITS;
    digit_mask &= RADIX - 1;  // the kernels' shared-memory tables hold RADIX digits
    upsweep<BITS><<<tiles, BLOCK, 0, s>>>(kin, n, shift, digit_mask, counts, totals, tiles);
    mark("radix_upsweep");
    scan_rows<<<RADIX, SCAN_BLOCK, 0, s>>>(counts, totals, tiles);
    mark("radix_scan");
    downsweep<BITS><<<tiles, BLOCK, WARPS * RADIX * sizeof(uint32_t), s>>>(
        kin, vin, kout, vout, n, shift, digit_mask, counts, tiles, rank_out);
    mark("radix_downsweep");
}

// Scratch words the sort needs for n keys: the count matrix plus per-pass digit totals.
inline size_t scratch_words(int n) {
    return (size_t)MAX_RADIX * num_tiles(n) + (size_t)MAX_PASSES * MAX_RADIX;
}

// Sorts (k0, v0) by the low plan bits, ping-ponging with (k1, v1); all four buffers hold n words.
// With `index_payload` the input payload is each key's index and v0 is not read.  The result
// buffers are returned through keys_out / vals_out.  With `rank_out` (n words), the last pass
// also writes rank_out[payload] = output position.  `mark(name)` is called after every kernel.
template <class Mark>
inline void sort_pairs(cudaStream_t s, const Plan& plan, uint32_t* k0, uint32_t* v0, uint32_t* k1,
                       uint32_t* v1, bool index_payload, uint32_t* scratch, int n,
                       uint32_t** keys_out, uint32_t** vals_out, Mark& mark,
                       uint32_t* rank_out = nullptr) {
    uint32_t* counts = scratch;
    uint32_t* totals = scratch + (size_t)MAX_RADIX * num_tiles(n);
    cudaMemsetAsync(totals, 0, sizeof(uint32_t) * MAX_PASSES * MAX_RADIX, s);
    const uint32_t* kin = k0;
    const uint32_t* vin = index_payload ? nullptr : v0;
    uint32_t* kout = k1;
    uint32_t* vout = v1;
    for (int p = 0; p < plan.passes; ++p) {
        uint32_t* tot = totals + (size_t)p * MAX_RADIX;
        const bool last = p + 1 == plan.passes;
        // a digit narrower than 8 bits only occurs in the last pass, where the key's higher
        // bits are zero, so the 8-bit kernel sorts it correctly
        if (plan.width[p] <= 8)
            run_pass<8>(s, kin, vin, kout, vout, counts, tot, n, plan.shift[p], last ? rank_out : nullptr, mark);
        else if (plan.width[p] == 9)
            run_pass<9>(s, kin, vin, kout, vout, counts, tot, n, plan.shift[p], last ? rank_out : nullptr, mark);
        else
            run_pass<10>(s, kin, vin, kout, vout, counts, tot, n, plan.shift[p], last ? rank_out : nullptr, mark);
        if (kout == k1) {
            kin = k1; vin = v1; kout = k0; vout = v0;
        } else {
            kin = k0; vin = v0; kout = k1; vout = v1;
        }
    }
    *keys_out = const_cast<uint32_t*>(kin);
    *vals_out = const_cast<uint32_t*>(vin);
}

}  // namespace radix
}  // namespace akua
