// Kernels of one PBF step.
//
// Two orders of the particles exist in a step:
//   * the reference order: particles sorted by cell hash, ties by the previous reference order —
//     exactly the order the reference leaves its buffer in (thrust::sort of whole records by hash,
//     NeighbourSearchCUDA.cu:167-170).  Bucket starts, the neighbour walk and the output records
//     follow it.
//   * the internal order: particles sorted by the Morton code of their cell, so that a warp's
//     particles and their neighbours sit close together in memory.  All per-particle state and the
//     neighbour passes use it.
// Results do not depend on the internal order: every per-particle sum runs over the neighbour list
// in the reference's walk order.
//
// Reference stages (paths relative to the AkuaEngine tree) and the kernels that cover them:
//   predict              IntegrationCUDA.cu:27-36            k_keys, k_gather
//   cell hash            NeighbourSearchCUDA.cu:15-44        k_keys
//   sort by hash         NeighbourSearchCUDA.cu:167-170      radix sort of (hash, previous rank)
//   bucket starts        NeighbourSearchCUDA.cu:52-65        k_ref, k_bucket_len
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
//   the particle in the reference order; nbr[k * n + i] = k-th neighbour of i (internal index);
//   xref[r] = (predicted position, mass) in reference order, Kr[r] = its hash.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pbf_device.cuh"

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

__global__ void k_set_params(StepParams p, StepParams* __restrict__ dst) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = p;
}

// Reads the attached records (buffer order = previous reference order) into the state.  A block
// stages its records through shared memory so global reads are coalesced when records are packed.
// With `carry`, density, lambda and position_delta are read too: with zero solver iterations the
// reference leaves them as they were.
__global__ void __launch_bounds__(kIoBlock)
    k_import(const char* __restrict__ aos, uint64_t stride, int n, float4* __restrict__ x4,
             float4* __restrict__ v4, float4* __restrict__ col4, float* __restrict__ size,
             uint32_t* __restrict__ rref, float* __restrict__ rho, float* __restrict__ lam,
             float4* __restrict__ dp4, int carry) {
    __shared__ float rec[kIoBlock * kRecWords];
    const int r0 = blockIdx.x * kIoBlock;
    const int cnt = min(kIoBlock, n - r0);
    if (stride == kRecWords * 4) {
        const float* src = reinterpret_cast<const float*>(aos) + (size_t)r0 * kRecWords;
        for (int w = threadIdx.x; w < cnt * kRecWords; w += kIoBlock) rec[w] = src[w];
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
    x4[i] = make_float4(r[kPos], r[kPos + 1], r[kPos + 2], r[kMass]);
    v4[i] = make_float4(r[kVel], r[kVel + 1], r[kVel + 2], 0.f);
    col4[i] = make_float4(r[kColor], r[kColor + 1], r[kColor + 2], r[kColor + 3]);
    size[i] = r[kSize];
    rref[i] = (uint32_t)i;
    if (carry) {
        rho[i] = r[kDensity];
        lam[i] = r[kLambda];
        dp4[i] = make_float4(r[kDelta], r[kDelta + 1], r[kDelta + 2], 0.f);
    }
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

// Cell hash of the predicted position, scattered into the previous reference order so the stable
// sort ties like the reference's; plus the Morton key of the walk cell.
__global__ void __launch_bounds__(kElemBlock)
    k_keys(const StepParams* __restrict__ P, const float4* __restrict__ x4,
           const float4* __restrict__ v4, const uint32_t* __restrict__ rref,
           uint32_t* __restrict__ akey, uint32_t* __restrict__ aval, uint32_t* __restrict__ skey) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float3 xs = predict(p, x4[i], v4[i]);
    const uint32_t h = cell_hash(cell_coord(xs.x, p.hash_cell), cell_coord(xs.y, p.hash_cell),
                                 cell_coord(xs.z, p.hash_cell), p.table_size, p.table_magic);
    const uint32_t r = rref[i];
    akey[r] = h;
    aval[r] = (uint32_t)i;
    skey[i] = morton_key(p, cell_coord(xs.x, p.search_cell), cell_coord(xs.y, p.search_cell),
                         cell_coord(xs.z, p.search_cell));
}

// Moves the state into the new internal order and writes the predicted positions.
// inv[old index] = new index.
__global__ void __launch_bounds__(kElemBlock)
    k_gather(const StepParams* __restrict__ P, const uint32_t* __restrict__ perm,
             const float4* __restrict__ x4, const float4* __restrict__ v4,
             const float4* __restrict__ col4, const float* __restrict__ size,
             float4* __restrict__ x4g, float4* __restrict__ col4g, float* __restrict__ sizeg,
             float4* __restrict__ ps0, uint32_t* __restrict__ inv,
             const float* __restrict__ rho_in, const float* __restrict__ lam_in,
             const float4* __restrict__ dp_in, float* __restrict__ rho_out,
             float* __restrict__ lam_out, float4* __restrict__ dp_out, int carry) {
    const StepParams& p = *P;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const uint32_t o = perm[s];
    const float4 x = x4[o];
    const float3 xs = predict(p, x, v4[o]);
    x4g[s] = x;
    col4g[s] = col4[o];
    sizeg[s] = size[o];
    ps0[s] = make_float4(xs.x, xs.y, xs.z, x.w);
    inv[o] = (uint32_t)s;
    if (carry) {
        rho_out[s] = rho_in[o];
        lam_out[s] = lam_in[o];
        dp_out[s] = dp_in[o];
    }
}

// Per reference rank r: internal index, reference-ordered predicted positions, the next step's
// reference rank of each particle, and the bucket starts: table[hash] = first rank carrying it
// (NeighbourSearchCUDA.cu:52-65).  The table is never cleared; a lookup is valid only if the rank
// it names still carries the looked-up hash, which holds exactly for this step's hashes.
__global__ void __launch_bounds__(kElemBlock)
    k_ref(const StepParams* __restrict__ P, const uint32_t* __restrict__ kr,
          const uint32_t* __restrict__ refperm, const uint32_t* __restrict__ inv,
          const float4* __restrict__ ps0, const uint32_t* __restrict__ rref_old,
          uint32_t* __restrict__ r2i, uint32_t* __restrict__ rref_new, float4* __restrict__ xref,
          uint32_t* __restrict__ table, uint32_t* __restrict__ order_out) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= P->n) return;
    const uint32_t o = refperm[r];
    const uint32_t s = inv[o];
    r2i[r] = s;
    rref_new[s] = (uint32_t)r;
    xref[r] = ps0[s];
    order_out[r] = rref_old[o];
    const uint32_t k = kr[r];
    if (r == 0 || kr[r - 1] != k) table[k] = (uint32_t)r;
}

// blen[start rank of a bucket] = number of ranks carrying its hash.
__global__ void __launch_bounds__(kElemBlock)
    k_bucket_len(const StepParams* __restrict__ P, const uint32_t* __restrict__ kr,
                 const uint32_t* __restrict__ table, uint32_t* __restrict__ blen) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = P->n;
    if (r >= n) return;
    const uint32_t k = kr[r];
    if (r == n - 1 || kr[r + 1] != k) {
        const uint32_t start = table[k];
        blen[start] = (uint32_t)r + 1u - start;
    }
}

// Accumulators of the density and lambda of one particle (ConstraintSolverCUDA.cu:16-97).  Kept
// separate as in the reference's two kernels, so the sums have the reference's order.
template <bool EXACT>
struct DensityLambda {
    float rho, gx, gy, gz, sum;
    __device__ __forceinline__ void init(float mi, const StepParams& p) {
        rho = mi * p.w0;
        gx = gy = gz = sum = 0.f;
    }
    __device__ __forceinline__ void add(const StepParams& p, float sx, float sy, float sz, float mj) {
        rho = __fmaf_rn(mj, poly6(p, len2(sx, sy, sz)), rho);
        const float3 g = spiky_grad<EXACT>(p, sx, sy, sz);
        gx = __fmaf_rn(mj, g.x, gx);
        gy = __fmaf_rn(mj, g.y, gy);
        gz = __fmaf_rn(mj, g.z, gz);
        const float s = (-p.inv_rho0) * mj;
        const float jx = s * g.x, jy = s * g.y, jz = s * g.z;
        sum = sum + len2(jx, jy, jz);
    }
    __device__ __forceinline__ float lambda(const StepParams& p) const {
        const float ax = gx * p.inv_rho0, ay = gy * p.inv_rho0, az = gz * p.inv_rho0;
        const float c = __fmaf_rn(rho, p.inv_rho0, -1.0f);
        const float den = (sum + len2(ax, ay, az)) + p.relaxation;
        return EXACT ? __fdiv_rn(-c, den) : __fdividef(-c, den);
    }
};

// Neighbour walk (NeighbourSearchCUDA.cu:72-130) in the reference's order: the 27 cells with dx
// outer and dz inner, each bucket in reference order, skipping self, accepting
// |x_i - x_j|^2 < h^2, stopping at the capacity.  The 27 bucket lookups are issued before the walk.
// When `density` is set, the first Jacobi iteration's density and lambda are accumulated on the
// way (same terms, same order).
template <bool EXACT>
__global__ void __launch_bounds__(kPairBlock)
    k_search(const StepParams* __restrict__ P, const float4* __restrict__ ps,
             const float4* __restrict__ xref, const uint32_t* __restrict__ kr,
             const uint32_t* __restrict__ table, const uint32_t* __restrict__ blen,
             const uint32_t* __restrict__ r2i, const uint32_t* __restrict__ rank_of,
             uint32_t* __restrict__ nbr, uint32_t* __restrict__ cnt, float* __restrict__ rho_out,
             float* __restrict__ lam_out, uint32_t* __restrict__ flags, int density) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = ps[i];
    const uint32_t ri = rank_of[i];
    const int cx = cell_coord(xi.x, p.search_cell);
    const int cy = cell_coord(xi.y, p.search_cell);
    const int cz = cell_coord(xi.z, p.search_cell);
    uint32_t hh[27], st[27];
#pragma unroll
    for (int d = 0; d < 27; ++d) {
        hh[d] = cell_hash(cx + d / 9 - 1, cy + (d / 3) % 3 - 1, cz + d % 3 - 1, p.table_size,
                          p.table_magic);
        st[d] = __ldg(table + hh[d]);
    }
#pragma unroll
    for (int d = 0; d < 27; ++d) {
        const uint32_t k = st[d];
        uint32_t len = 0u, start = 0u;
        if (k < (uint32_t)n) {
            if (__ldg(kr + k) == hh[d]) {
                len = __ldg(blen + k);
                start = k;
            }
        }
        hh[d] = len;  // from here on: bucket length
        st[d] = start;
    }
    const int cap = p.cap;
    uint32_t* col = nbr + i;
    int count = 0;
    DensityLambda<EXACT> acc;
    acc.init(xi.w, p);
    for (int d = 0; d < 27 && count < cap; ++d) {
        const uint32_t end = st[d] + hh[d];
        for (uint32_t r = st[d]; r < end; ++r) {
            if (r == ri) continue;
            const float4 xj = __ldg(xref + r);
            const float sx = xi.x - xj.x, sy = xi.y - xj.y, sz = xi.z - xj.z;
            if (len2(sx, sy, sz) < p.h2) {
                col[(size_t)count * n] = __ldg(r2i + r);
                if (density) acc.add(p, sx, sy, sz, xj.w);
                if (++count == cap) break;
            }
        }
    }
    cnt[i] = (uint32_t)count;
    if (count >= cap) atomicOr(flags, kFlagCapReached);
    if (density) {
        rho_out[i] = acc.rho;
        lam_out[i] = acc.lambda(p);
    }
}

template <bool EXACT>
__global__ void __launch_bounds__(kPairBlock)
    k_density_lambda(const StepParams* __restrict__ P, const float4* __restrict__ ps,
                     const uint32_t* __restrict__ nbr, const uint32_t* __restrict__ cnt,
                     float* __restrict__ rho_out, float* __restrict__ lam_out) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = ps[i];
    const uint32_t* col = nbr + i;
    const int c = (int)cnt[i];
    DensityLambda<EXACT> acc;
    acc.init(xi.w, p);
#pragma unroll 4
    for (int k = 0; k < c; ++k) {
        const float4 xj = __ldg(ps + __ldg(col + (size_t)k * n));
        acc.add(p, xi.x - xj.x, xi.y - xj.y, xi.z - xj.z, xj.w);
    }
    rho_out[i] = acc.rho;
    lam_out[i] = acc.lambda(p);
}

// Position delta with artificial pressure (ConstraintSolverCUDA.cu:99-130).
template <bool EXACT>
__device__ __forceinline__ float3 position_delta(const StepParams& p, int n, float4 xi, float li,
                                                 const float4* __restrict__ ps,
                                                 const float* __restrict__ lam,
                                                 const uint32_t* __restrict__ col, int c) {
    float dx = 0.f, dy = 0.f, dz = 0.f;
#pragma unroll 4
    for (int k = 0; k < c; ++k) {
        const uint32_t j = __ldg(col + (size_t)k * n);
        const float4 xj = __ldg(ps + j);
        const float lj = __ldg(lam + j);
        const float sx = xi.x - xj.x, sy = xi.y - xj.y, sz = xi.z - xj.z;
        const float sc = scorr<EXACT>(p, len2(sx, sy, sz));
        const float b = ((li + lj) + sc) * xj.w;
        const float3 g = spiky_grad<EXACT>(p, sx, sy, sz);
        dx = __fmaf_rn(b, g.x, dx);
        dy = __fmaf_rn(b, g.y, dy);
        dz = __fmaf_rn(b, g.z, dz);
    }
    return make_float3(dx * p.inv_rho0, dy * p.inv_rho0, dz * p.inv_rho0);
}

// Soft box clamp of one coordinate (ConstraintSolverCUDA.cu:136-157).
__device__ __forceinline__ float clamp_axis(float x, float lo_wall, float hi_wall) {
    const float lo = lo_wall + 0.025f, hi = hi_wall - 0.025f;
    float c = 0.f;
    if (x < lo) c = __fmaf_rn(0.5f, lo - x, c);
    if (x > hi) c = __fmaf_rn(0.5f, hi - x, c);
    return x + c;
}

template <bool EXACT>
__global__ void __launch_bounds__(kPairBlock)
    k_delta_correct(const StepParams* __restrict__ P, const float4* __restrict__ ps_in,
                    const float* __restrict__ lam, const uint32_t* __restrict__ nbr,
                    const uint32_t* __restrict__ cnt, float4* __restrict__ ps_out,
                    float4* __restrict__ dp4) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 xi = ps_in[i];
    const float3 d = position_delta<EXACT>(p, p.n, xi, lam[i], ps_in, lam, nbr + i, (int)cnt[i]);
    dp4[i] = make_float4(d.x, d.y, d.z, 0.f);
    ps_out[i] = make_float4(clamp_axis(xi.x + d.x, p.box_min[0], p.box_max[0]),
                            clamp_axis(xi.y + d.y, p.box_min[1], p.box_max[1]),
                            clamp_axis(xi.z + d.z, p.box_min[2], p.box_max[2]), xi.w);
}

// resolve_collision against one axis-aligned plane (IntegrationCUDA.cu:51-73), with the plane
// given as the reference builds it (IntegrationCUDA.cu:90-97): point on one axis, unit normal.
__device__ __forceinline__ void damp_plane(const StepParams& p, float px, float py, float pz,
                                           float qx, float qy, float qz, float nx, float ny, float nz,
                                           float& vx, float& vy, float& vz) {
    const float dist = dot3(px - qx, py - qy, pz - qz, nx, ny, nz);
    const float appr = dot3(vx, vy, vz, nx, ny, nz);
    if (dist < 0.025f) {
        const float vnx = appr * nx, vny = appr * ny, vnz = appr * nz;
        const float tx = vx - vnx, ty = vy - vny, tz = vz - vnz;
        if (appr < 0.0f) {
            vx = __fmaf_rn(p.neg_restitution, vnx, p.keep * tx);
            vy = __fmaf_rn(p.neg_restitution, vny, p.keep * ty);
            vz = __fmaf_rn(p.neg_restitution, vnz, p.keep * tz);
        } else if (fabsf(appr) < 1e-5f) {
            vx = p.keep * tx;
            vy = p.keep * ty;
            vz = p.keep * tz;
        }
    }
}

// Last Jacobi iteration fused with update (IntegrationCUDA.cu:38-49) and boundary damping
// (IntegrationCUDA.cu:75-102).  With `has_delta == 0` (zero iterations) the predicted positions
// go straight to the update.  Also moves the gathered colour, size, reference rank and (with
// `carry`) density/lambda/delta into the state arrays.
template <bool EXACT>
__global__ void __launch_bounds__(kPairBlock)
    k_delta_final(const StepParams* __restrict__ P, const float4* __restrict__ ps_in,
                  const float* __restrict__ lam, const uint32_t* __restrict__ nbr,
                  const uint32_t* __restrict__ cnt, const float4* __restrict__ x_old,
                  float4* __restrict__ x4, float4* __restrict__ v4, float4* __restrict__ vstar4,
                  float4* __restrict__ dp4, const float4* __restrict__ col4g,
                  const float* __restrict__ sizeg, float4* __restrict__ col4,
                  float* __restrict__ size, const uint32_t* __restrict__ rref_new,
                  uint32_t* __restrict__ rref, const float* __restrict__ rho_c,
                  const float* __restrict__ lam_c, const float4* __restrict__ dp_c,
                  float* __restrict__ rho, float* __restrict__ lam_out, int has_delta) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 xi = ps_in[i];
    float nx = xi.x, ny = xi.y, nz = xi.z;
    if (has_delta) {
        const float3 d = position_delta<EXACT>(p, p.n, xi, lam[i], ps_in, lam, nbr + i, (int)cnt[i]);
        dp4[i] = make_float4(d.x, d.y, d.z, 0.f);
        nx = clamp_axis(xi.x + d.x, p.box_min[0], p.box_max[0]);
        ny = clamp_axis(xi.y + d.y, p.box_min[1], p.box_max[1]);
        nz = clamp_axis(xi.z + d.z, p.box_min[2], p.box_max[2]);
    } else {
        rho[i] = rho_c[i];
        lam_out[i] = lam_c[i];
        dp4[i] = dp_c[i];
    }
    const float4 xo = x_old[i];
    const float vx0 = __fdiv_rn(nx - xo.x, p.dt);
    const float vy0 = __fdiv_rn(ny - xo.y, p.dt);
    const float vz0 = __fdiv_rn(nz - xo.z, p.dt);
    vstar4[i] = make_float4(vx0, vy0, vz0, 0.f);
    float vx = vx0, vy = vy0, vz = vz0;
    damp_plane(p, nx, ny, nz, p.box_min[0], 0.f, 0.f, 1.f, 0.f, 0.f, vx, vy, vz);
    damp_plane(p, nx, ny, nz, p.box_max[0], 0.f, 0.f, -1.f, 0.f, 0.f, vx, vy, vz);
    damp_plane(p, nx, ny, nz, 0.f, p.box_min[1], 0.f, 0.f, 1.f, 0.f, vx, vy, vz);
    damp_plane(p, nx, ny, nz, 0.f, p.box_max[1], 0.f, 0.f, -1.f, 0.f, vx, vy, vz);
    damp_plane(p, nx, ny, nz, 0.f, 0.f, p.box_min[2], 0.f, 0.f, 1.f, vx, vy, vz);
    damp_plane(p, nx, ny, nz, 0.f, 0.f, p.box_max[2], 0.f, 0.f, -1.f, vx, vy, vz);
    x4[i] = make_float4(nx, ny, nz, xi.w);
    v4[i] = make_float4(vx, vy, vz, 0.f);
    col4[i] = col4g[i];
    size[i] = sizeg[i];
    rref[i] = rref_new[i];
}

// omega_i = sum_j -m_j (v_j - v_i) x grad W(x_i - x_j)  (IntegrationCUDA.cu:104-128).
// om4.w = |omega_i| for the confinement pass.
template <bool EXACT>
__global__ void __launch_bounds__(kPairBlock)
    k_vorticity(const StepParams* __restrict__ P, const float4* __restrict__ x4,
                const float4* __restrict__ v4, const uint32_t* __restrict__ nbr,
                const uint32_t* __restrict__ cnt, float4* __restrict__ om4) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = x4[i], vi = v4[i];
    const uint32_t* col = nbr + i;
    const int c = (int)cnt[i];
    float wx = 0.f, wy = 0.f, wz = 0.f;
#pragma unroll 4
    for (int k = 0; k < c; ++k) {
        const uint32_t j = __ldg(col + (size_t)k * n);
        const float4 xj = __ldg(x4 + j), vj = __ldg(v4 + j);
        const float3 g = spiky_grad<EXACT>(p, xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        const float3 cr = cross3(vj.x - vi.x, vj.y - vi.y, vj.z - vi.z, g.x, g.y, g.z);
        const float s = -xj.w;
        wx = __fmaf_rn(s, cr.x, wx);
        wy = __fmaf_rn(s, cr.y, wy);
        wz = __fmaf_rn(s, cr.z, wz);
    }
    om4[i] = make_float4(wx, wy, wz, __fsqrt_rn(len2(wx, wy, wz)));
}

// Vorticity confinement (IntegrationCUDA.cu:130-165); writes the confined velocity to a separate
// buffer with vc4.w = m_i / rho_i for the XSPH pass.
template <bool EXACT>
__global__ void __launch_bounds__(kPairBlock)
    k_confine(const StepParams* __restrict__ P, const float4* __restrict__ x4,
              const float4* __restrict__ v4, const float4* __restrict__ om4,
              const float* __restrict__ rho, const uint32_t* __restrict__ nbr,
              const uint32_t* __restrict__ cnt, float4* __restrict__ vc4) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = x4[i], vi = v4[i], wi = om4[i];
    const float rho_i = rho[i];
    const uint32_t* col = nbr + i;
    const int c = (int)cnt[i];
    float ex = 0.f, ey = 0.f, ez = 0.f;
#pragma unroll 4
    for (int k = 0; k < c; ++k) {
        const uint32_t j = __ldg(col + (size_t)k * n);
        const float4 xj = __ldg(x4 + j);
        const float s = xj.w * (wi.w - __ldg(&om4[j].w));
        const float3 g = spiky_grad<EXACT>(p, xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
        ex = __fmaf_rn(s, g.x, ex);
        ey = __fmaf_rn(s, g.y, ey);
        ez = __fmaf_rn(s, g.z, ez);
    }
    const float inv_d = __fdiv_rn(1.0f, rho_i);
    ex = ex * inv_d;
    ey = ey * inv_d;
    ez = ez * inv_d;
    float vx = vi.x, vy = vi.y, vz = vi.z;
    const float el = __fsqrt_rn(len2(ex, ey, ez));
    if (!(el < 1e-5f)) {
        float nx, ny, nz;
        if (EXACT) {
            nx = __fdiv_rn(ex, el); ny = __fdiv_rn(ey, el); nz = __fdiv_rn(ez, el);
        } else {
            const float inv = __fdividef(1.0f, el);
            nx = ex * inv; ny = ey * inv; nz = ez * inv;
        }
        const float3 cr = cross3(nx, ny, nz, wi.x, wi.y, wi.z);
        vx = __fmaf_rn(p.dt, p.vort_eps * cr.x, vx);
        vy = __fmaf_rn(p.dt, p.vort_eps * cr.y, vy);
        vz = __fmaf_rn(p.dt, p.vort_eps * cr.z, vz);
    }
    vc4[i] = make_float4(vx, vy, vz, __fdiv_rn(xi.w, rho_i));
}

// XSPH viscosity (IntegrationCUDA.cu:167-195) from the confined-velocity snapshot vc4.
__global__ void __launch_bounds__(kPairBlock)
    k_xsph(const StepParams* __restrict__ P, const float4* __restrict__ x4,
           const float4* __restrict__ vc4, const uint32_t* __restrict__ nbr,
           const uint32_t* __restrict__ cnt, float4* __restrict__ v4) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = x4[i], vi = vc4[i];
    const uint32_t* col = nbr + i;
    const int c = (int)cnt[i];
    float ax = 0.f, ay = 0.f, az = 0.f;
#pragma unroll 4
    for (int k = 0; k < c; ++k) {
        const uint32_t j = __ldg(col + (size_t)k * n);
        const float4 xj = __ldg(x4 + j), vj = __ldg(vc4 + j);
        const float w = poly6(p, len2(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z));
        const float tx = vj.w * (vj.x - vi.x), ty = vj.w * (vj.y - vi.y), tz = vj.w * (vj.z - vi.z);
        ax = __fmaf_rn(tx, w, ax);
        ay = __fmaf_rn(ty, w, ay);
        az = __fmaf_rn(tz, w, az);
    }
    v4[i] = make_float4(__fmaf_rn(p.visc, ax, vi.x), __fmaf_rn(p.visc, ay, vi.y),
                        __fmaf_rn(p.visc, az, vi.z), 0.f);
}

// Writes every field of every particle into the attached records in reference order (record r
// holds the particle of reference rank r), staged through shared memory so global writes are
// coalesced when records are packed.
__global__ void __launch_bounds__(kIoBlock)
    k_export(char* __restrict__ aos, uint64_t stride, int n, const uint32_t* __restrict__ r2i,
             const uint32_t* __restrict__ kr, const float4* __restrict__ x4,
             const float4* __restrict__ v4, const float4* __restrict__ vstar4,
             const float4* __restrict__ dp4, const float4* __restrict__ om4,
             const float* __restrict__ rho, const float* __restrict__ lam,
             const float4* __restrict__ col4, const float* __restrict__ size) {
    __shared__ float rec[kIoBlock * kRecWords];
    const int r0 = blockIdx.x * kIoBlock;
    const int cnt = min(kIoBlock, n - r0);
    const int t = threadIdx.x;
    if (t < cnt) {
        const int r = r0 + t;
        const uint32_t s = r2i[r];
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
        o[kHash] = __uint_as_float(kr[r]);
        o[kColor] = c.x; o[kColor + 1] = c.y; o[kColor + 2] = c.z; o[kColor + 3] = c.w;
        o[kSize] = size[s];
    }
    __syncthreads();
    if (stride == kRecWords * 4) {
        float* dst = reinterpret_cast<float*>(aos) + (size_t)r0 * kRecWords;
        for (int w = t; w < cnt * kRecWords; w += kIoBlock) dst[w] = rec[w];
    } else {
        for (int w = t; w < cnt * kRecWords; w += kIoBlock) {
            const int q = w / kRecWords, f = w - q * kRecWords;
            reinterpret_cast<float*>(aos + (uint64_t)(r0 + q) * stride)[f] = rec[w];
        }
    }
}

}  // namespace akua
