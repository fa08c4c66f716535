// Kernels of one PBF step.
//
// Two orders of the particles exist in a step:
//   * the reference order: particles sorted by cell hash, ties by the previous reference order —
//     exactly the order the reference leaves its buffer in (thrust::sort of whole records by hash,
//     NeighbourSearchCUDA.cu:167-170).  Bucket starts, the neighbour walk and the output records
//     follow it.
//   * the internal order: particles sorted by the Morton code of their cell, so that a warp's
//     particles and their neighbours sit close together in memory.  All per-particle state and the
//     neighbour passes use it.  It is a stable sort over the previous reference order, so it does
//     not wait for the hash sort: particles of one cell share their hash, so their order within
//     the cell is their new reference order either way (cells that share a clamped Morton key
//     and are not contiguous are found by k_table_build and walked by rank).
// Results do not depend on the internal order: every per-particle sum runs over the neighbour list
// in the reference's walk order.
//
// Reference stages (paths relative to the AkuaEngine tree) and the kernels that cover them:
//   predict              IntegrationCUDA.cu:27-36            k_import or k_keys, k_gather
//   cell hash            NeighbourSearchCUDA.cu:15-44        k_import or k_keys (write_keys)
//   sort by hash         NeighbourSearchCUDA.cu:167-170      radix sort of (hash, previous rank)
//   bucket starts        NeighbourSearchCUDA.cu:52-65        k_table_build
//   neighbour walk       NeighbourSearchCUDA.cu:72-130       k_search (+ iteration 1 density/lambda)
//   density, lambda      ConstraintSolverCUDA.cu:16-97       k_search / k_density_lambda
//   delta, correct       ConstraintSolverCUDA.cu:99-169      k_delta_correct / k_delta_final
//   update, damping      IntegrationCUDA.cu:38-102           k_delta_final
//   vorticity            IntegrationCUDA.cu:104-128          k_vorticity
//   confinement          IntegrationCUDA.cu:130-165          k_confine
//   XSPH                 IntegrationCUDA.cu:167-195          k_xsph (reads a velocity snapshot)
//
// Layout (internal order unless noted):
//   x4 = (position, mass), v4 = (velocity, 0), ps[b] = (predicted position, mass), rref = rank of
//   the particle in the reference order; neighbour lists in uint4 tiles (pbf_pairs.cuh) of
//   internal indices; xref[r] = (predicted position, mass) in reference order, Kr[r] = its hash.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pbf_device.cuh"
#include "pbf_pairs.cuh"
#include "pbf_search.cuh"

namespace akua {

constexpr int kElemBlock = 256;
constexpr int kPairBlock = 128;
constexpr int kIoBlock = 128;

enum : uint32_t { kFlagCapReached = 1u, kFlagBadTable = 2u };

// Word offsets inside one 108-byte particle record (Particle.h:8-31).
enum RecWord : int {
    kPos = 0, kVel = 3, kNewPos = 6, kNewVel = 9, kDelta = 12, kVort = 15,
    kMass = 18, kDensity = 19, kLambda = 20, kHash = 21, kColor = 22, kSize = 26, kRecWords = 27
};

// Block-wide copy of `words` floats, in 16-byte pieces when both ends allow it (a block of
// kIoBlock packed 108-byte records starts on a 16-byte boundary of a 16-byte aligned array); the
// records may live in host memory read over the host link, where wide accesses matter most.
__device__ __forceinline__ void copy_words(float* __restrict__ dst, const float* __restrict__ src,
                                           int words) {
    int done = 0;
    if ((((uintptr_t)dst | (uintptr_t)src) & 15u) == 0) {
        const int vec = words >> 2;
        const uint4* s4 = reinterpret_cast<const uint4*>(src);
        uint4* d4 = reinterpret_cast<uint4*>(dst);
        for (int w = threadIdx.x; w < vec; w += blockDim.x) d4[w] = s4[w];
        done = vec << 2;
    }
    for (int w = done + threadIdx.x; w < words; w += blockDim.x) dst[w] = src[w];
}

__global__ void k_set_params(StepParams p, StepParams* __restrict__ dst) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = p;
}

// Per-scene parameters of a batch, uploaded in chunks passed by value (kernel parameters are
// captured at launch, so the host copy may change right after).
constexpr int kParamChunk = 16;  // 16 x 168 bytes: under the classic 4 KB parameter limit
struct ParamChunk {
    StepParams p[kParamChunk];
    int count;
};
__global__ void k_set_params_chunk(ParamChunk c, StepParams* __restrict__ dst) {
    if (blockIdx.x == 0 && threadIdx.x < c.count) dst[threadIdx.x] = c.p[threadIdx.x];
}


// Predicted position (IntegrationCUDA.cu:34-35): v* = fma(g, dt, v); x* = fma(v*, dt, x).
__device__ __forceinline__ float3 predict(const StepParams& p, float4 x, float4 v) {
    const float vx = __fmaf_rn(p.gravity[0], p.dt, v.x);
    const float vy = __fmaf_rn(p.gravity[1], p.dt, v.y);
    const float vz = __fmaf_rn(p.gravity[2], p.dt, v.z);
    return make_float3(__fmaf_rn(vx, p.dt, x.x), __fmaf_rn(vy, p.dt, x.y), __fmaf_rn(vz, p.dt, x.z));
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Morton code of a cell relative to the box's lowest cell, each axis clamped to sp_bits bits.
// Only memory locality depends on it.
__device__ __forceinline__ uint32_t morton_key(const StepParams& p, int cx, int cy, int cz) {
    const int hi = (1 << p.sp_bits) - 1;
    const uint32_t x = (uint32_t)min(max(cx - p.sp_origin[0], 0), hi);
    const uint32_t y = (uint32_t)min(max(cy - p.sp_origin[1], 0), hi);
    const uint32_t z = (uint32_t)min(max(cz - p.sp_origin[2], 0), hi);
    return spread10(x) | (spread10(y) << 1) | (spread10(z) << 2);
}

// Hash key and Morton key of the predicted position of import slot i at previous reference rank r.
__device__ __forceinline__ void write_keys(const StepParams& p, float4 x, float4 v, uint32_t r,
                                           uint32_t i, uint32_t* __restrict__ akey,
                                           uint32_t* __restrict__ aval, uint32_t* __restrict__ bkey,
                                           uint32_t* __restrict__ bval) {
    const float3 xs = predict(p, x, v);
    const uint32_t h = cell_hash(cell_coord(xs.x, p.hash_cell), cell_coord(xs.y, p.hash_cell),
                                 cell_coord(xs.z, p.hash_cell), p.table_size, p.table_magic);
    akey[r] = p.table_offset + h;
    aval[r] = i;
    bkey[r] = ((uint32_t)p.scene << (3 * p.sp_bits)) |
              morton_key(p, cell_coord(xs.x, p.search_cell), cell_coord(xs.y, p.search_cell),
                         cell_coord(xs.z, p.search_cell));
    bval[r] = i;
}

// Cell hash and Morton key of the walk cell of each predicted position, both scattered into the
// previous reference order (so both stable sorts tie like the reference's), each with the import
// index as payload.  Steps that import the records compute them in k_import instead.
__global__ void __launch_bounds__(kElemBlock)
    k_keys(const StepParams* __restrict__ P, const float4* __restrict__ x4,
           const float4* __restrict__ v4, const uint32_t* __restrict__ rref,
           uint32_t* __restrict__ akey, uint32_t* __restrict__ aval, uint32_t* __restrict__ bkey,
           uint32_t* __restrict__ bval) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P->n) return;
    write_keys(params_for(P, i), x4[i], v4[i], rref[i], (uint32_t)i, akey, aval, bkey, bval);
}

// Reads the attached records (buffer order = previous reference order) into the state, and writes
// the sort keys as k_keys does (an import slot's previous reference rank is its index).  A block
// stages its records through shared memory so global reads are coalesced when records are packed.
// With `carry`, density, lambda and position_delta are read too: with zero solver iterations the
// reference leaves them as they were.
__global__ void __launch_bounds__(kIoBlock)
    k_import(const StepParams* __restrict__ P, const char* __restrict__ aos, uint64_t stride,
             int n, float4* __restrict__ x4, float4* __restrict__ v4, float4* __restrict__ col4,
             float* __restrict__ size, uint32_t* __restrict__ rref, float* __restrict__ rho,
             float* __restrict__ lam, float4* __restrict__ dp4, int carry,
             uint32_t* __restrict__ akey, uint32_t* __restrict__ aval, uint32_t* __restrict__ bkey,
             uint32_t* __restrict__ bval) {
    __shared__ __align__(16) float rec[kIoBlock * kRecWords];
    const int r0 = blockIdx.x * kIoBlock;
    const int cnt = min(kIoBlock, n - r0);
    if (stride == kRecWords * 4) {
        const float* src = reinterpret_cast<const float*>(aos) + (size_t)r0 * kRecWords;
        copy_words(rec, src, cnt * kRecWords);
    } else {
        for (int w = threadIdx.x; w < cnt * kRecWords; w += kIoBlock) {
            const int q = w / kRecWords, f = w - q * kRecWords;
            rec[w] = reinterpret_cast<const float*>(aos + (uint64_t)(r0 + q) * stride)[f];
        }
    }
    __syncthreads();
    const int t = threadIdx.x;
    if (t >= cnt) return;
    const int i = r0 + t;
    const float* r = rec + t * kRecWords;
    const float4 x = make_float4(r[kPos], r[kPos + 1], r[kPos + 2], r[kMass]);
    const float4 v = make_float4(r[kVel], r[kVel + 1], r[kVel + 2], 0.f);
    x4[i] = x;
    v4[i] = v;
    write_keys(params_for(P, i), x, v, (uint32_t)i, (uint32_t)i, akey, aval, bkey, bval);
    col4[i] = make_float4(r[kColor], r[kColor + 1], r[kColor + 2], r[kColor + 3]);
    size[i] = r[kSize];
    rref[i] = (uint32_t)i;
    if (carry) {
        rho[i] = r[kDensity];
        lam[i] = r[kLambda];
        dp4[i] = make_float4(r[kDelta], r[kDelta + 1], r[kDelta + 2], 0.f);
    }
}


// Moves the state into the new internal order (slot s holds the particle of import index
// sp_import[s], reference rank rank_of_import[...]) and writes the predicted positions, both maps
// between ranks and slots, the reference-ordered predicted positions and the debug order
// (pre-sort record index per rank).
__global__ void __launch_bounds__(kElemBlock)
    k_gather(const StepParams* __restrict__ P, const uint32_t* __restrict__ sp_import,
             const uint32_t* __restrict__ rank_of_import, const float4* __restrict__ x4,
             const float4* __restrict__ v4, const float4* __restrict__ col4,
             const float* __restrict__ size, const uint32_t* __restrict__ rref_old,
             float4* __restrict__ x4g, float4* __restrict__ col4g, float* __restrict__ sizeg,
             float4* __restrict__ ps0, uint32_t* __restrict__ r2i, uint32_t* __restrict__ rank_of,
             float4* __restrict__ xref, uint32_t* __restrict__ order_out,
             const float* __restrict__ rho_in, const float* __restrict__ lam_in,
             const float4* __restrict__ dp_in, float* __restrict__ rho_out,
             float* __restrict__ lam_out, float4* __restrict__ dp_out, int carry,
             const float* __restrict__ lacc_src, float* __restrict__ lprev_out,
             float* __restrict__ speed_out, uint32_t* __restrict__ mass_bits) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    // masses: mass_bits[0] stays 0 while every mass has the bit pattern of record 0, which
    // mass_bits[1] holds; a warp that sees another pattern sets mass_bits[0] once
    const uint32_t ref_bits = __float_as_uint(__ldg(&x4[0].w));
    bool other = false;
    if (s < P->n) {
        const StepParams& p = params_for(P, s);
        const uint32_t o = sp_import[s];       // import index of internal slot s
        const uint32_t r = rank_of_import[o];  // its new reference rank
        const float4 x = x4[o];
        const float4 v = v4[o];
        const float3 xs = predict(p, x, v);
        if (speed_out) {  // learned modes: |predicted velocity| and last step's accumulated lambda
            const float vx = __fmaf_rn(p.gravity[0], p.dt, v.x);
            const float vy = __fmaf_rn(p.gravity[1], p.dt, v.y);
            const float vz = __fmaf_rn(p.gravity[2], p.dt, v.z);
            speed_out[s] = sqrtf(vx * vx + vy * vy + vz * vz);
            lprev_out[s] = lacc_src[o];
        }
        const float4 q = make_float4(xs.x, xs.y, xs.z, x.w);
        x4g[s] = x;
        col4g[s] = col4[o];
        sizeg[s] = size[o];
        ps0[s] = q;
        r2i[r] = (uint32_t)s;
        rank_of[s] = r;
        xref[r] = q;
        order_out[r] = rref_old[o];
        if (carry) {
            rho_out[s] = rho_in[o];
            lam_out[s] = lam_in[o];
            dp_out[s] = dp_in[o];
        }
        other = __float_as_uint(x.w) != ref_bits;
        if (s == 0) mass_bits[1] = ref_bits;
    }
    if (__any_sync(0xFFFFFFFFu, other) && (threadIdx.x & 31) == 0) atomicOr(mass_bits, 1u);
}

// The bucket table (NeighbourSearchCUDA.cu:52-65 builds hash -> first sorted index).  Here an
// entry is (x, y): y = 0 for a hash no particle carries; otherwise y = bucket length and x = the
// bucket's first internal slot, or, with bit 31 of y set (a mixed bucket, see k_table_build), its
// first reference rank.  The table is all-empty between steps: k_xsph empties this step's
// entries after the walk.

// One thread per bucket start (the first reference rank carrying a hash) reads its bucket's ranks
// (a short run of the sorted keys) and writes the entry: the length, and whether the bucket's
// particles are one contiguous run of internal slots in rank order (then x = the first slot) or
// not (several cells share the hash, or clamped cells share a Morton key: x = the first rank,
// mixed bit set).
__global__ void __launch_bounds__(kElemBlock)
    k_table_build(const StepParams* __restrict__ P, const uint32_t* __restrict__ kr,
                  const uint32_t* __restrict__ r2i, uint2* __restrict__ table) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = P->n;
    if (r >= n) return;
    const uint32_t k = kr[r];
    if (r > 0 && kr[r - 1] == k) return;
    const uint32_t s0 = r2i[r];
    uint32_t prev = s0;
    bool run = true;
    int e = r + 1;
    for (; e < n && kr[e] == k; ++e) {
        const uint32_t se = r2i[e];
        run = run && se == prev + 1u;
        prev = se;
    }
    const uint32_t len = (uint32_t)(e - r);
    table[k] = run ? make_uint2(s0, len) : make_uint2((uint32_t)r, len | kMixedBucket);
}


// Writes every field of every particle into the attached records in reference order (record r
// holds the particle of reference rank r), staged through shared memory so global writes are
// coalesced when records are packed.
__global__ void __launch_bounds__(kIoBlock)
    k_export(const StepParams* __restrict__ P, char* __restrict__ aos, uint64_t stride, int n,
             const uint32_t* __restrict__ r2i,
             const uint32_t* __restrict__ kr, const float4* __restrict__ x4,
             const float4* __restrict__ v4, const float4* __restrict__ vstar4,
             const float4* __restrict__ dp4, const float4* __restrict__ om4,
             const float* __restrict__ rho, const float* __restrict__ lam,
             const float4* __restrict__ col4, const float* __restrict__ size,
             const float* __restrict__ lacc, float* __restrict__ lacc_ref) {
    __shared__ __align__(16) float rec[kIoBlock * kRecWords];
    const int r0 = blockIdx.x * kIoBlock;
    const int cnt = min(kIoBlock, n - r0);
    const int t = threadIdx.x;
    if (t < cnt) {
        const int r = r0 + t;
        const uint32_t s = r2i[r];
        if (lacc_ref) lacc_ref[r] = lacc[s];
        const float4 x = x4[s], v = v4[s], vs = vstar4[s], d = dp4[s], w = om4[s], c = col4[s];
        float* o = rec + t * kRecWords;
        o[kPos] = x.x; o[kPos + 1] = x.y; o[kPos + 2] = x.z;
        o[kVel] = v.x; o[kVel + 1] = v.y; o[kVel + 2] = v.z;
        o[kNewPos] = x.x; o[kNewPos + 1] = x.y; o[kNewPos + 2] = x.z;
        o[kNewVel] = vs.x; o[kNewVel + 1] = vs.y; o[kNewVel + 2] = vs.z;
        o[kDelta] = d.x; o[kDelta + 1] = d.y; o[kDelta + 2] = d.z;
        o[kVort] = w.x; o[kVort + 1] = w.y; o[kVort + 2] = w.z;
        o[kMass] = x.w;
        o[kDensity] = rho[s];
        o[kLambda] = lam[s];
        o[kHash] = __uint_as_float(kr[r] - params_for(P, r).table_offset);  // the scene's own hash
        o[kColor] = c.x; o[kColor + 1] = c.y; o[kColor + 2] = c.z; o[kColor + 3] = c.w;
        o[kSize] = size[s];
    }
    __syncthreads();
    if (stride == kRecWords * 4) {
        float* dst = reinterpret_cast<float*>(aos) + (size_t)r0 * kRecWords;
        copy_words(dst, rec, cnt * kRecWords);
    } else {
        for (int w = t; w < cnt * kRecWords; w += kIoBlock) {
            const int q = w / kRecWords, f = w - q * kRecWords;
            reinterpret_cast<float*>(aos + (uint64_t)(r0 + q) * stride)[f] = rec[w];
        }
    }
}

}  // namespace akua
