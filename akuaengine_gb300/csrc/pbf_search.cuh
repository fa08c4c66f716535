// Neighbour walk of the PBF step (NeighbourSearchCUDA.cu:72-130).
//
// The reference's walk: for the 27 cells around a particle's cell (dx outer, dz inner), look up
// the bucket of the cell's hash — a run of the hash-sorted (reference) order — and walk it in that
// order, skipping self, accepting |x_i - x_j|^2 < h^2, until maxNeighbours entries are found.  A
// bucket shared by two of the 27 cells is walked twice.
//
// The internal order sorts particles by the Morton code of their cell and, inside a cell, by
// reference rank.  A bucket that holds one cell is therefore a contiguous run of internal slots in
// the same order the reference walks it: a candidate's slot is directly its list entry.  Buckets
// flagged as mixed (several cells on one hash, or cells sharing a clamped Morton key) are read in
// reference order through the reference-ordered positions, their ranks mapped to slots.  Both give
// the reference's list, entry for entry.
//
// Warp-cooperative walk.  A warp takes 32 consecutive particles; consecutive particles of the same
// cell (a run) share one candidate sequence: the concatenation of the 27 buckets in walk order.
// For each run, lanes 0..26 look up one bucket each and a warp scan gives each bucket's offset in
// the sequence.  The sequence is then read 32 candidates at a time, one per lane (coalesced: the
// buckets are contiguous runs), and every particle of the run tests the whole chunk at once; a
// ballot and a population count place each hit at the particle's running count plus the hits of
// lower lanes, which is the reference's order.  Each candidate is loaded once per run instead of
// once per particle, and no lane idles on another lane's bucket length.  Two particles are tested
// per round (independent ballots and placements, distances in packed FP32x2): their dependency
// chains interleave, which a lane-serial walk or a windowed one (both measured slower) cannot.
//
// The first STAGE entries of each list are staged in shared memory and written out as coalesced
// uint4 tiles (pbf_pairs.cuh).  The block size and STAGE (the walk's tile shape) are template
// parameters; the solver's autotuner picks them by measurement (lists do not depend on them).
// When `density` is set, the first Jacobi iteration's density and lambda are accumulated over the
// finished list, one thread per particle (same terms, same order as k_density_lambda).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pbf_device.cuh"
#include "pbf_learned.cuh"
#include "pbf_pairs.cuh"

namespace akua {

constexpr int kSearchBlock = 128;  // default tile shape: 128 threads, 32 staged entries
constexpr int kListStage = 32;
// Row stride in words of STAGE staged entries: STAGE + 4 words, an odd number of 16-byte units
// (9 for 32, 5 for 16), so the uint4 rows of a warp's lanes fall in different banks.
__host__ __device__ constexpr int list_row(int stage) { return stage + 4; }
__host__ __device__ constexpr size_t search_smem(int block, int stage) {
    return sizeof(uint32_t) * block * list_row(stage) + sizeof(float4) * block;
}
constexpr size_t kSearchSmem = search_smem(kSearchBlock, kListStage);
constexpr uint32_t kFullWarp = 0xffffffffu;
constexpr uint32_t kMixedBucket = 0x80000000u;  // bucket table: y bit for a mixed bucket
constexpr uint32_t kDenseRun = 2048;  // candidates of a run beyond which the walk may stop early

template <bool EXACT, int BLOCK, int STAGE>
__global__ void __launch_bounds__(BLOCK)
    k_search(const StepParams* __restrict__ P, const float4* __restrict__ ps,
             const float4* __restrict__ xref, const uint2* __restrict__ table,
             const uint32_t* __restrict__ r2i, uint32_t* __restrict__ nbr,
             uint32_t* __restrict__ cnt, float* __restrict__ rho_out, float* __restrict__ lam_out,
             uint32_t* __restrict__ flags, int density, const float* __restrict__ speed,
             const float* __restrict__ lprev, float* __restrict__ lacc,
             float* __restrict__ feat, float4* __restrict__ psl) {
    extern __shared__ __align__(16) uint32_t stage[];
    const StepParams& p = *P;
    const int n = p.n;
    const int lane = threadIdx.x & 31;
    const int wbase = threadIdx.x & ~31;
    constexpr int kListRow = list_row(STAGE);
    const int base = blockIdx.x * BLOCK + wbase;  // this warp's first particle
    if (base >= n) return;                               // uniform over the warp
    const int i = base + lane;
    const bool valid = i < n;
    float4* xs = reinterpret_cast<float4*>(stage + BLOCK * kListRow) + wbase;
    uint32_t* rows = stage + wbase * kListRow;

    const float4 xi = valid ? ps[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    xs[lane] = xi;
    const int cx = cell_coord(xi.x, p.search_cell);
    const int cy = cell_coord(xi.y, p.search_cell);
    const int cz = cell_coord(xi.z, p.search_cell);
    // a run: consecutive particles of one scene in one cell
    const int sid = (valid && p.scene_of) ? (int)p.scene_of[i] : 0;
    const int px = __shfl_up_sync(kFullWarp, cx, 1);
    const int py = __shfl_up_sync(kFullWarp, cy, 1);
    const int pz = __shfl_up_sync(kFullWarp, cz, 1);
    const int ps_ = __shfl_up_sync(kFullWarp, sid, 1);
    uint32_t starts = __ballot_sync(
        kFullWarp, valid && (lane == 0 || px != cx || py != cy || pz != cz || ps_ != sid));
    const int nvalid = min(32, n - base);
    __syncwarp();

    const float h2 = p.h2;
    const int cap = p.cap;
    const uint32_t below = (1u << lane) - 1u;
    int count = 0;  // lane q: running list length of particle base + q
    while (starts) {
        const int q0 = __ffs(starts) - 1;
        starts &= starts - 1;
        const int q1 = starts ? __ffs(starts) - 1 : nvalid;
        const int rx = __shfl_sync(kFullWarp, cx, q0);
        const int ry = __shfl_sync(kFullWarp, cy, q0);
        const int rz = __shfl_sync(kFullWarp, cz, q0);
        const StepParams& pr = P[__shfl_sync(kFullWarp, sid, q0)];  // the run's scene
        // lane b < 27 holds bucket b of the walk (dx = b/9 - 1, dy = b/3%3 - 1, dz = b%3 - 1)
        uint2 e = make_uint2(0u, 0u);
        if (lane < 27)
            e = __ldg(table + pr.table_offset +
                      cell_hash(rx + lane / 9 - 1, ry + lane / 3 % 3 - 1, rz + lane % 3 - 1,
                                pr.table_size, pr.table_magic));
        const uint32_t blen = e.y & ~kMixedBucket;
        uint32_t incl = blen;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(kFullWarp, incl, o);
            if (lane >= o) incl += v;
        }
        const uint32_t off = incl - blen;  // lanes 27..31: the sequence length
        const uint32_t total = __shfl_sync(kFullWarp, incl, 31);

        // one chunk of 32 candidates of the run's sequence
        auto chunk = [&](uint32_t c0) {
            const uint32_t at = c0 + lane;
            int b = 0;  // the last bucket starting at or before `at`
#pragma unroll
            for (int step = 16; step; step >>= 1)
                if (__shfl_sync(kFullWarp, off, b + step) <= at) b += step;
            const uint32_t bx = __shfl_sync(kFullWarp, e.x, b);
            const uint32_t by = __shfl_sync(kFullWarp, e.y, b);
            const uint32_t bo = __shfl_sync(kFullWarp, off, b);
            const bool live = at < total;
            float4 c = make_float4(__int_as_float(0x7f800000), __int_as_float(0x7f800000),
                                   __int_as_float(0x7f800000), 0.f);
            uint32_t j = 0xffffffffu;
            if (live) {
                const uint32_t t = bx + (at - bo);
                if (by & kMixedBucket) {
                    c = __ldg(xref + t);
                    j = __ldg(r2i + t);
                } else {
                    c = __ldg(ps + t);
                    j = t;
                }
            }
            // two particles per round: independent tests, ballots and placements
            const uint32_t jrel = j - (uint32_t)base;  // == q for particle q's own slot
            const float2 cxx = f2(c.x), cyy = f2(c.y), czz = f2(c.z);
            auto place = [&](int q, int pos) {
                if (pos < STAGE) rows[q * kListRow + pos] = j;
                else if (pos < cap) nbr[4 * ((size_t)(pos >> 2) * n + base + q) + (pos & 3)] = j;
            };
            int q = q0;
            for (; q + 1 < q1; q += 2) {
                const float4 xa = xs[q], xb = xs[q + 1];
                const float2 d2 = len2_2(sub2(make_float2(xa.x, xb.x), cxx),
                                         sub2(make_float2(xa.y, xb.y), cyy),
                                         sub2(make_float2(xa.z, xb.z), czz));
                const bool ha = d2.x < h2 && jrel != (uint32_t)q;
                const bool hb = d2.y < h2 && jrel != (uint32_t)(q + 1);
                const uint32_t ba = __ballot_sync(kFullWarp, ha);
                const uint32_t bb = __ballot_sync(kFullWarp, hb);
                const int pa = __shfl_sync(kFullWarp, count, q) + __popc(ba & below);
                const int pb = __shfl_sync(kFullWarp, count, q + 1) + __popc(bb & below);
                if (ha) place(q, pa);
                if (hb) place(q + 1, pb);
                count += lane == q ? __popc(ba) : (lane == q + 1 ? __popc(bb) : 0);
            }
            if (q < q1) {
                const float4 xq = xs[q];
                const bool hit = len2(xq.x - c.x, xq.y - c.y, xq.z - c.z) < h2 && jrel != (uint32_t)q;
                const uint32_t bal = __ballot_sync(kFullWarp, hit);
                const int pos = __shfl_sync(kFullWarp, count, q) + __popc(bal & below);
                if (hit) place(q, pos);
                if (lane == q) count += __popc(bal);
            }
        };
        if (total <= kDenseRun) {
            for (uint32_t c0 = 0; c0 < total; c0 += 32) chunk(c0);
        } else {
            // a pile-up far denser than any cell of a resting fluid: stop once every list of the
            // run is full (later hits are neither stored nor needed for the overflow flag; a list
            // fills only after at least cap candidates), or such a run would cost run size x
            // sequence length tests
            for (uint32_t c0 = 0; c0 < total; c0 += 32) {
                if (c0 >= (uint32_t)cap &&
                    __all_sync(kFullWarp, lane < q0 || lane >= q1 || count >= cap))
                    break;
                chunk(c0);
            }
        }
    }
    __syncwarp();
    if (!valid) return;
    const int total_count = count;
    count = count < cap ? count : cap;
    cnt[i] = (uint32_t)count;
    if (total_count >= cap) atomicOr(flags, 1u);
    const uint32_t* myrow = rows + lane * kListRow;

    // staged entries -> global tiles (a partial last tile carries unused words)
    const int staged = min(count, STAGE);
    const uint4* row4 = reinterpret_cast<const uint4*>(myrow);
    uint4* out4 = reinterpret_cast<uint4*>(nbr);
    for (int g = 0; g < (staged + 3) >> 2; ++g) out4[(size_t)g * n + i] = row4[g];

    // first iteration's density and lambda over the finished list, read in uint4 tiles (staged
    // rows are conflict-free that way)
    if (density) {
        DensityLambda2<EXACT> acc;
        acc.init(xi.w, p);
        const uint4* tiles = reinterpret_cast<const uint4*>(nbr) + i;
        for (int g = 0; 4 * g < count; ++g) {
            const uint4 e = g < STAGE / 4 ? row4[g] : tiles[(size_t)g * n];
            const int left = count - 4 * g;
            acc.add2(p, xi, __ldg(ps + e.x), __ldg(ps + (left >= 2 ? e.y : e.x)), left >= 2);
            if (left > 2)
                acc.add2(p, xi, __ldg(ps + e.z), __ldg(ps + (left >= 4 ? e.w : e.z)), left >= 4);
        }
        rho_out[i] = acc.rho;
        const float l = acc.lambda(p);
        lam_out[i] = l;
        psl[i] = make_float4(xi.x, xi.y, xi.z, l);
        if (feat) {  // learned modes: the lambda sum starts; the network's features
            lacc[i] = l;
            write_features(params_for(P, i), acc, l, count, lprev[i], speed[i],
                           feat + (size_t)kFeatures * i);
        }
    }
}

}  // namespace akua
