// Kernels of one PBF step over structure-of-arrays particle state in hash-sorted order.
//
// Reference stages (paths relative to the AkuaEngine tree) and the kernel that covers each:
//   predict              IntegrationCUDA.cu:27-36            k_predict_hash, k_gather (recomputed)
//   cell hash            NeighbourSearchCUDA.cu:15-44        k_predict_hash
//   sort by hash         NeighbourSearchCUDA.cu:167-170      radix::sort_pairs + k_gather
//   bucket starts        NeighbourSearchCUDA.cu:52-65        k_build_table
//   neighbour walk       NeighbourSearchCUDA.cu:72-130       k_search (+ iteration 1 density/lambda)
//   density              ConstraintSolverCUDA.cu:16-42       k_search / k_density_lambda
//   lambda               ConstraintSolverCUDA.cu:51-97       k_search / k_density_lambda
//   position delta       ConstraintSolverCUDA.cu:99-130      k_delta_correct / k_delta_final
//   correct + clamp      ConstraintSolverCUDA.cu:136-169     k_delta_correct / k_delta_final
//   update               IntegrationCUDA.cu:38-49            k_delta_final
//   boundary damping     IntegrationCUDA.cu:51-102           k_delta_final
//   vorticity            IntegrationCUDA.cu:104-128          k_vorticity
//   confinement          IntegrationCUDA.cu:130-165          k_confine
//   XSPH                 IntegrationCUDA.cu:167-195          k_xsph (reads a velocity snapshot)
//
// Layout (all in hash-sorted order after k_gather):
//   x4[i]    = (position, mass)            v4[i]  = (velocity, 0)
//   ps[b][i] = (predicted position, mass)  double-buffered across Jacobi iterations
//   nbr[i * cap + k] = k-th neighbour of i (the reference's row layout), cnt[i] = list length
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pbf_device.cuh"

namespace akua {

constexpr int kElemBlock = 256;
constexpr int kPairBlock = 128;

enum : uint32_t { kFlagCapReached = 1u, kFlagBadTable = 2u };

// Word offsets inside one 108-byte particle record (Particle.h:8-31).
enum RecWord : int {
    kPos = 0, kVel = 3, kNewPos = 6, kNewVel = 9, kDelta = 12, kVort = 15,
    kMass = 18, kDensity = 19, kLambda = 20, kHash = 21, kColor = 22, kSize = 26, kRecWords = 27
};

__global__ void k_set_params(StepParams p, StepParams* __restrict__ dst) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = p;
}

// Reads the attached records into SoA state (buffer order).  With `carry`, density, lambda and
// position_delta are read too: with zero solver iterations the reference leaves them untouched.
__global__ void __launch_bounds__(kElemBlock)
    k_import(const char* __restrict__ aos, uint64_t stride, int n, float4* __restrict__ x4,
             float4* __restrict__ v4, float4* __restrict__ col4, float* __restrict__ size,
             float* __restrict__ rho, float* __restrict__ lam, float4* __restrict__ dp4, int carry) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = reinterpret_cast<const float*>(aos + (uint64_t)i * stride);
    x4[i] = make_float4(r[kPos], r[kPos + 1], r[kPos + 2], r[kMass]);
    v4[i] = make_float4(r[kVel], r[kVel + 1], r[kVel + 2], 0.f);
    col4[i] = make_float4(r[kColor], r[kColor + 1], r[kColor + 2], r[kColor + 3]);
    size[i] = r[kSize];
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

__global__ void __launch_bounds__(kElemBlock)
    k_predict_hash(const StepParams* __restrict__ P, const float4* __restrict__ x4,
                   const float4* __restrict__ v4, uint32_t* __restrict__ keys) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float3 xs = predict(p, x4[i], v4[i]);
    keys[i] = cell_hash(cell_coord(xs.x, p.hash_cell), cell_coord(xs.y, p.hash_cell),
                        cell_coord(xs.z, p.hash_cell), p.table_size);
}

// Moves the state into sorted order and writes the predicted positions.
__global__ void __launch_bounds__(kElemBlock)
    k_gather(const StepParams* __restrict__ P, const uint32_t* __restrict__ perm,
             const float4* __restrict__ x4, const float4* __restrict__ v4,
             const float4* __restrict__ col4, const float* __restrict__ size,
             float4* __restrict__ x4g, float4* __restrict__ v4g, float4* __restrict__ col4g,
             float* __restrict__ sizeg, float4* __restrict__ ps0, const float* __restrict__ rho_in,
             const float* __restrict__ lam_in, const float4* __restrict__ dp_in,
             float* __restrict__ rho_out, float* __restrict__ lam_out, float4* __restrict__ dp_out,
             int carry) {
    const StepParams& p = *P;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= p.n) return;
    const uint32_t src = perm[s];
    const float4 x = x4[src];
    const float4 v = v4[src];
    x4g[s] = x;
    v4g[s] = v;
    col4g[s] = col4[src];
    sizeg[s] = size[src];
    const float3 xs = predict(p, x, v);
    ps0[s] = make_float4(xs.x, xs.y, xs.z, x.w);
    if (carry) {
        rho_out[s] = rho_in[src];
        lam_out[s] = lam_in[src];
        dp_out[s] = dp_in[src];
    }
}

// table[hash] = first sorted slot carrying that hash (NeighbourSearchCUDA.cu:52-65).  The table is
// never cleared: a lookup is valid only if the slot it names still carries the looked-up hash,
// which holds exactly for the hashes present in this step.
__global__ void __launch_bounds__(kElemBlock)
    k_build_table(const StepParams* __restrict__ P, const uint32_t* __restrict__ keys,
                  uint32_t* __restrict__ table) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P->n) return;
    const uint32_t k = keys[s];
    if (s == 0 || keys[s - 1] != k) table[k] = (uint32_t)s;
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

// Neighbour walk over the 27 cells (NeighbourSearchCUDA.cu:72-130), in the reference's order
// (dx outer, dz inner; bucket order within a cell), skipping self, stopping at the bucket end,
// accepting |x_i - x_j|^2 < h^2 and stopping at the capacity.  When `density` is set the first
// Jacobi iteration's density and lambda are accumulated on the way (same terms, same order).
template <bool EXACT>
__global__ void __launch_bounds__(kPairBlock)
    k_search(const StepParams* __restrict__ P, const float4* __restrict__ ps,
             const uint32_t* __restrict__ keys, const uint32_t* __restrict__ table,
             uint32_t* __restrict__ nbr, uint32_t* __restrict__ cnt, float* __restrict__ rho_out,
             float* __restrict__ lam_out, uint32_t* __restrict__ flags, int density) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = ps[i];
    const int cx = cell_coord(xi.x, p.search_cell);
    const int cy = cell_coord(xi.y, p.search_cell);
    const int cz = cell_coord(xi.z, p.search_cell);
    const int cap = p.cap;
    uint32_t* row = nbr + (size_t)i * cap;
    int count = 0;
    DensityLambda<EXACT> acc;
    acc.init(xi.w, p);
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                const uint32_t hh = cell_hash(cx + dx, cy + dy, cz + dz, p.table_size);
                int k = (int)table[hh];
                if (k < 0 || k >= n || keys[k] != hh) continue;
                while (k < n && count < cap) {
                    if (k == i) { ++k; continue; }
                    if (keys[k] != hh) break;
                    const float4 xj = ps[k];
                    const float sx = xi.x - xj.x, sy = xi.y - xj.y, sz = xi.z - xj.z;
                    if (len2(sx, sy, sz) < p.h2) {
                        row[count++] = (uint32_t)k;
                        if (density) acc.add(p, sx, sy, sz, xj.w);
                    }
                    ++k;
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
    if (i >= p.n) return;
    const float4 xi = ps[i];
    const uint32_t* row = nbr + (size_t)i * p.cap;
    const int c = (int)cnt[i];
    DensityLambda<EXACT> acc;
    acc.init(xi.w, p);
    for (int k = 0; k < c; ++k) {
        const float4 xj = ps[row[k]];
        acc.add(p, xi.x - xj.x, xi.y - xj.y, xi.z - xj.z, xj.w);
    }
    rho_out[i] = acc.rho;
    lam_out[i] = acc.lambda(p);
}

// Position delta with artificial pressure (ConstraintSolverCUDA.cu:99-130).
template <bool EXACT>
__device__ __forceinline__ float3 position_delta(const StepParams& p, int i, float4 xi, float li,
                                                 const float4* __restrict__ ps,
                                                 const float* __restrict__ lam,
                                                 const uint32_t* __restrict__ row, int c) {
    float dx = 0.f, dy = 0.f, dz = 0.f;
    for (int k = 0; k < c; ++k) {
        const uint32_t j = row[k];
        const float4 xj = ps[j];
        const float sx = xi.x - xj.x, sy = xi.y - xj.y, sz = xi.z - xj.z;
        const float sc = scorr<EXACT>(p, len2(sx, sy, sz));
        const float b = ((li + lam[j]) + sc) * xj.w;
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
    const float3 d = position_delta<EXACT>(p, i, xi, lam[i], ps_in, lam, nbr + (size_t)i * p.cap,
                                           (int)cnt[i]);
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
// go straight to the update.  Also moves the sorted colour/size back into the state arrays.
template <bool EXACT>
__global__ void __launch_bounds__(kPairBlock)
    k_delta_final(const StepParams* __restrict__ P, const float4* __restrict__ ps_in,
                  const float* __restrict__ lam, const uint32_t* __restrict__ nbr,
                  const uint32_t* __restrict__ cnt, const float4* __restrict__ x_old,
                  float4* __restrict__ x4, float4* __restrict__ v4, float4* __restrict__ vstar4,
                  float4* __restrict__ dp4, const float4* __restrict__ col4g,
                  const float* __restrict__ sizeg, float4* __restrict__ col4,
                  float* __restrict__ size, int has_delta) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    const float4 xi = ps_in[i];
    float nx = xi.x, ny = xi.y, nz = xi.z;
    if (has_delta) {
        const float3 d = position_delta<EXACT>(p, i, xi, lam[i], ps_in, lam,
                                               nbr + (size_t)i * p.cap, (int)cnt[i]);
        dp4[i] = make_float4(d.x, d.y, d.z, 0.f);
        nx = clamp_axis(xi.x + d.x, p.box_min[0], p.box_max[0]);
        ny = clamp_axis(xi.y + d.y, p.box_min[1], p.box_max[1]);
        nz = clamp_axis(xi.z + d.z, p.box_min[2], p.box_max[2]);
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
    if (i >= p.n) return;
    const float4 xi = x4[i], vi = v4[i];
    const uint32_t* row = nbr + (size_t)i * p.cap;
    const int c = (int)cnt[i];
    float wx = 0.f, wy = 0.f, wz = 0.f;
    for (int k = 0; k < c; ++k) {
        const uint32_t j = row[k];
        const float4 xj = x4[j], vj = v4[j];
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
    if (i >= p.n) return;
    const float4 xi = x4[i], vi = v4[i], wi = om4[i];
    const float rho_i = rho[i];
    const uint32_t* row = nbr + (size_t)i * p.cap;
    const int c = (int)cnt[i];
    float ex = 0.f, ey = 0.f, ez = 0.f;
    for (int k = 0; k < c; ++k) {
        const uint32_t j = row[k];
        const float4 xj = x4[j];
        const float s = xj.w * (wi.w - om4[j].w);
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
    if (i >= p.n) return;
    const float4 xi = x4[i], vi = vc4[i];
    const uint32_t* row = nbr + (size_t)i * p.cap;
    const int c = (int)cnt[i];
    float ax = 0.f, ay = 0.f, az = 0.f;
    for (int k = 0; k < c; ++k) {
        const uint32_t j = row[k];
        const float4 xj = x4[j], vj = vc4[j];
        const float w = poly6(p, len2(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z));
        const float tx = vj.w * (vj.x - vi.x), ty = vj.w * (vj.y - vi.y), tz = vj.w * (vj.z - vi.z);
        ax = __fmaf_rn(tx, w, ax);
        ay = __fmaf_rn(ty, w, ay);
        az = __fmaf_rn(tz, w, az);
    }
    v4[i] = make_float4(__fmaf_rn(p.visc, ax, vi.x), __fmaf_rn(p.visc, ay, vi.y),
                        __fmaf_rn(p.visc, az, vi.z), 0.f);
}

// Writes every field of the sorted particles back into the attached records.
__global__ void __launch_bounds__(kElemBlock)
    k_export(char* __restrict__ aos, uint64_t stride, int n, const float4* __restrict__ x4,
             const float4* __restrict__ v4, const float4* __restrict__ vstar4,
             const float4* __restrict__ dp4, const float4* __restrict__ om4,
             const float* __restrict__ rho, const float* __restrict__ lam,
             const uint32_t* __restrict__ keys, const float4* __restrict__ col4,
             const float* __restrict__ size) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float* r = reinterpret_cast<float*>(aos + (uint64_t)i * stride);
    const float4 x = x4[i], v = v4[i], vs = vstar4[i], d = dp4[i], w = om4[i], c = col4[i];
    r[kPos] = x.x; r[kPos + 1] = x.y; r[kPos + 2] = x.z;
    r[kVel] = v.x; r[kVel + 1] = v.y; r[kVel + 2] = v.z;
    r[kNewPos] = x.x; r[kNewPos + 1] = x.y; r[kNewPos + 2] = x.z;
    r[kNewVel] = vs.x; r[kNewVel + 1] = vs.y; r[kNewVel + 2] = vs.z;
    r[kDelta] = d.x; r[kDelta + 1] = d.y; r[kDelta + 2] = d.z;
    r[kVort] = w.x; r[kVort + 1] = w.y; r[kVort + 2] = w.z;
    r[kMass] = x.w;
    r[kDensity] = rho[i];
    r[kLambda] = lam[i];
    reinterpret_cast<uint32_t*>(r)[kHash] = keys[i];
    r[kColor] = c.x; r[kColor + 1] = c.y; r[kColor + 2] = c.z; r[kColor + 3] = c.w;
    r[kSize] = size[i];
}

}  // namespace akua
