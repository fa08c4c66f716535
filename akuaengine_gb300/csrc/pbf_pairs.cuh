// Neighbour-pair passes of the PBF step, evaluated two neighbours at a time with Blackwell's packed
// FP32 instructions (__fadd2_rn / __fmul2_rn / __ffma2_rn: two IEEE round-to-nearest operations in
// one instruction).  Each lane of a packed operation rounds exactly like the scalar operation, so a
// pair term is bit-identical to its scalar evaluation; the per-particle sums stay scalar and run
// in list order.
//
// Neighbour lists are stored as uint4 tiles: nbr4[g * n + i] holds entries 4g..4g+3 of particle i,
// so one coalesced 16-byte load per lane fetches four neighbour indices.  Entries at or beyond a
// particle's count are never dereferenced.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pbf_device.cuh"

namespace akua {

// The neighbour-pair kernels run with a block size chosen per kernel (64, 128 or 256 threads; the
// solver's autotuner picks them by measurement); results do not depend on it.
constexpr int kMaxPairBlock = 256;

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b: fma(b, -1, a) is the exact difference rounded once, i.e. the IEEE subtraction.
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// dot3 of each lane (same contraction as the scalar dot3)
__device__ __forceinline__ float2 len2_2(float2 x, float2 y, float2 z) {
    return fma2(z, z, fma2(x, x, mul2(y, y)));
}

__device__ __forceinline__ float2 poly6_2(const StepParams& p, float2 r2) {
    const float2 d = sub2(f2(p.h2), r2);
    const float2 w = mul2(f2(p.kp), mul2(mul2(d, d), d));
    return make_float2(r2.x > p.h2 ? 0.0f : w.x, r2.y > p.h2 ? 0.0f : w.y);
}

// Spiky gradient coefficient c with grad W = c * r (per lane).
template <bool EXACT>
__device__ __forceinline__ void spiky2(const StepParams& p, float2 sx, float2 sy, float2 sz,
                                       float2 r2, float2& gx, float2& gy, float2& gz) {
    if constexpr (EXACT) {
        const float rx = __fsqrt_rn(r2.x), ry = __fsqrt_rn(r2.y);
        const float2 q = sub2(f2(p.h), make_float2(rx, ry));
        const float2 c = mul2(f2(p.ks), mul2(q, q));
        const float2 ax = mul2(c, sx), ay = mul2(c, sy), az = mul2(c, sz);
        const bool zx = rx > p.h || rx < 1e-5f, zy = ry > p.h || ry < 1e-5f;
        gx = make_float2(zx ? 0.f : __fdiv_rn(ax.x, rx), zy ? 0.f : __fdiv_rn(ax.y, ry));
        gy = make_float2(zx ? 0.f : __fdiv_rn(ay.x, rx), zy ? 0.f : __fdiv_rn(ay.y, ry));
        gz = make_float2(zx ? 0.f : __fdiv_rn(az.x, rx), zy ? 0.f : __fdiv_rn(az.y, ry));
    } else {
        const float2 ir = make_float2(rsqrtf(r2.x), rsqrtf(r2.y));
        const float2 r = mul2(r2, ir);
        const float2 q = sub2(f2(p.h), r);
        float2 c = mul2(mul2(f2(p.ks), mul2(q, q)), ir);
        if (r2.x > p.h2 || r2.x < 1e-10f) c.x = 0.f;
        if (r2.y > p.h2 || r2.y < 1e-10f) c.y = 0.f;
        gx = mul2(c, sx);
        gy = mul2(c, sy);
        gz = mul2(c, sz);
    }
}

// Calls f(j0, j1, two) for consecutive neighbour pairs of one particle in list order; `two` is
// false only for a trailing single entry, in which case j1 == j0 and must not be accumulated.
// The next tile of indices is loaded while the current one is processed.
template <class F>
__device__ __forceinline__ void for_each_pair(const uint4* __restrict__ col, int n, int c, F&& f) {
    const int ng = (c + 3) >> 2;
    if (ng == 0) return;
    uint4 cur = __ldg(col);
    for (int g = 0; g < ng; ++g) {
        uint4 nxt = make_uint4(0u, 0u, 0u, 0u);
        if (g + 1 < ng) nxt = __ldg(col + (size_t)(g + 1) * n);
        const int left = c - 4 * g;
        f(cur.x, left >= 2 ? cur.y : cur.x, left >= 2);
        if (left > 2) f(cur.z, left >= 4 ? cur.w : cur.z, left >= 4);
        cur = nxt;
    }
}

// A particle's two-float4 record (x.xyz, w0 | v.xyz, w1) read in one 256-bit load (32-byte
// aligned: record j starts at float4 2j of a cudaMalloc'd array).
struct Rec8 {
    float4 x, v;
};
__device__ __forceinline__ Rec8 ld_rec8(const float4* __restrict__ rec, uint32_t j) {
    Rec8 r;
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(r.x.x), "=f"(r.x.y), "=f"(r.x.z), "=f"(r.x.w), "=f"(r.v.x), "=f"(r.v.y),
          "=f"(r.v.z), "=f"(r.v.w)
        : "l"(rec + 2 * (size_t)j));
    return r;
}

// Density and lambda accumulators (ConstraintSolverCUDA.cu:16-97), two neighbours per call.
template <bool EXACT>
struct DensityLambda2 {
    float rho, gx, gy, gz, sum;
    __device__ __forceinline__ void init(float mi, const StepParams& p) {
        rho = mi * p.w0;
        gx = gy = gz = sum = 0.f;
    }
    __device__ __forceinline__ void add2(const StepParams& p, float4 xi, float4 a, float4 b,
                                         bool two) {
        const float2 sx = sub2(f2(xi.x), make_float2(a.x, b.x));
        const float2 sy = sub2(f2(xi.y), make_float2(a.y, b.y));
        const float2 sz = sub2(f2(xi.z), make_float2(a.z, b.z));
        const float2 r2 = len2_2(sx, sy, sz);
        const float2 w = poly6_2(p, r2);
        float2 ux, uy, uz;
        spiky2<EXACT>(p, sx, sy, sz, r2, ux, uy, uz);
        const float2 s = mul2(f2(-p.inv_rho0), make_float2(a.w, b.w));
        const float2 l = len2_2(mul2(s, ux), mul2(s, uy), mul2(s, uz));
        rho = __fmaf_rn(a.w, w.x, rho);
        gx = __fmaf_rn(a.w, ux.x, gx);
        gy = __fmaf_rn(a.w, uy.x, gy);
        gz = __fmaf_rn(a.w, uz.x, gz);
        sum = sum + l.x;
        if (two) {
            rho = __fmaf_rn(b.w, w.y, rho);
            gx = __fmaf_rn(b.w, ux.y, gx);
            gy = __fmaf_rn(b.w, uy.y, gy);
            gz = __fmaf_rn(b.w, uz.y, gz);
            sum = sum + l.y;
        }
    }
    __device__ __forceinline__ float lambda(const StepParams& p) const {
        const float ax = gx * p.inv_rho0, ay = gy * p.inv_rho0, az = gz * p.inv_rho0;
        const float c = __fmaf_rn(rho, p.inv_rho0, -1.0f);
        const float den = (sum + len2(ax, ay, az)) + p.relaxation;
        return EXACT ? __fdiv_rn(-c, den) : __fdividef(-c, den);
    }
};

template <bool EXACT>
__global__ void __launch_bounds__(kMaxPairBlock)
    k_density_lambda(const StepParams* __restrict__ P, const float4* __restrict__ ps,
                     const uint4* __restrict__ nbr4, const uint32_t* __restrict__ cnt,
                     float* __restrict__ rho_out, float* __restrict__ lam_out,
                     float* __restrict__ lacc, float4* __restrict__ psl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P->n) return;
    const StepParams& p = params_for(P, i);
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = ps[i];
    DensityLambda2<EXACT> acc;
    acc.init(xi.w, p);
    for_each_pair(nbr4 + i, n, (int)cnt[i], [&](uint32_t j0, uint32_t j1, bool two) {
        acc.add2(p, xi, __ldg(ps + j0), __ldg(ps + j1), two);
    });
    rho_out[i] = acc.rho;
    const float l = acc.lambda(p);
    lam_out[i] = l;
    psl[i] = make_float4(xi.x, xi.y, xi.z, l);
    if (lacc) lacc[i] += l;  // learned modes: the step's accumulated lambda
}

// (W(r2) / W(dq^2))^n of two pairs: the power in s_corr = -k * (...)^n (ConstraintSolverCUDA.cu:124).
template <bool EXACT>
__device__ __forceinline__ float2 scorr_pow2(const StepParams& p, float2 r2) {
    const float2 w = poly6_2(p, r2);
    float2 ratio;
    if (EXACT) ratio = make_float2(__fdiv_rn(w.x, p.wdq), __fdiv_rn(w.y, p.wdq));
    else ratio = mul2(w, f2(p.inv_wdq));
    float2 pw;
    if (p.corr_n_int == 4) {
        const float2 q = mul2(ratio, ratio);
        pw = mul2(q, q);
    } else if (p.corr_n_int >= 0) {
        pw = make_float2(pown(ratio.x, p.corr_n_int), pown(ratio.y, p.corr_n_int));
    } else {
        pw = make_float2(powf(ratio.x, p.corr_n), powf(ratio.y, p.corr_n));
    }
    return pw;
}

// Position delta with artificial pressure (ConstraintSolverCUDA.cu:99-130).
template <bool EXACT>
__device__ __forceinline__ float3 position_delta(const StepParams& p, int n, float4 xi, float li,
                                                 const float4* __restrict__ ps,
                                                 const float* __restrict__ lam,
                                                 const uint4* __restrict__ col, int c) {
    float dx = 0.f, dy = 0.f, dz = 0.f;
    for_each_pair(col, n, c, [&](uint32_t j0, uint32_t j1, bool two) {
        const float4 a = __ldg(ps + j0), b = __ldg(ps + j1);
        const float2 lj = make_float2(__ldg(lam + j0), __ldg(lam + j1));
        const float2 sx = sub2(f2(xi.x), make_float2(a.x, b.x));
        const float2 sy = sub2(f2(xi.y), make_float2(a.y, b.y));
        const float2 sz = sub2(f2(xi.z), make_float2(a.z, b.z));
        const float2 r2 = len2_2(sx, sy, sz);
        // (lambda_i + lambda_j + s_corr) * m_j with s_corr = -k * pw: the product feeds the sum
        // and is contracted into it, as the CUDA compiler does with the reference's expression
        // (ConstraintSolverCUDA.cu:124-126).
        const float2 pw = scorr_pow2<EXACT>(p, r2);
        const float2 bb = mul2(fma2(f2(p.neg_k), pw, add2(f2(li), lj)), make_float2(a.w, b.w));
        float2 gx, gy, gz;
        spiky2<EXACT>(p, sx, sy, sz, r2, gx, gy, gz);
        dx = __fmaf_rn(bb.x, gx.x, dx);
        dy = __fmaf_rn(bb.x, gy.x, dy);
        dz = __fmaf_rn(bb.x, gz.x, dz);
        if (two) {
            dx = __fmaf_rn(bb.y, gx.y, dx);
            dy = __fmaf_rn(bb.y, gy.y, dy);
            dz = __fmaf_rn(bb.y, gz.y, dz);
        }
    });
    return make_float3(dx * p.inv_rho0, dy * p.inv_rho0, dz * p.inv_rho0);
}

// The same sum when every particle has mass `m`: positions and lambdas come from one 16-byte
// gather of psl[j] = (x*_j, lambda_j), and (lambda_i + lambda_j + s_corr) * m is the same product.
template <bool EXACT>
__device__ __forceinline__ float3 position_delta_uniform(const StepParams& p, int n, float4 xl,
                                                         const float4* __restrict__ psl, float m,
                                                         const uint4* __restrict__ col, int c) {
    float dx = 0.f, dy = 0.f, dz = 0.f;
    for_each_pair(col, n, c, [&](uint32_t j0, uint32_t j1, bool two) {
        const float4 a = __ldg(psl + j0), b = __ldg(psl + j1);
        const float2 sx = sub2(f2(xl.x), make_float2(a.x, b.x));
        const float2 sy = sub2(f2(xl.y), make_float2(a.y, b.y));
        const float2 sz = sub2(f2(xl.z), make_float2(a.z, b.z));
        const float2 r2 = len2_2(sx, sy, sz);
        const float2 pw = scorr_pow2<EXACT>(p, r2);
        const float2 bb = mul2(fma2(f2(p.neg_k), pw, add2(f2(xl.w), make_float2(a.w, b.w))), f2(m));
        float2 gx, gy, gz;
        spiky2<EXACT>(p, sx, sy, sz, r2, gx, gy, gz);
        dx = __fmaf_rn(bb.x, gx.x, dx);
        dy = __fmaf_rn(bb.x, gy.x, dy);
        dz = __fmaf_rn(bb.x, gz.x, dz);
        if (two) {
            dx = __fmaf_rn(bb.y, gx.y, dx);
            dy = __fmaf_rn(bb.y, gy.y, dy);
            dz = __fmaf_rn(bb.y, gz.y, dz);
        }
    });
    return make_float3(dx * p.inv_rho0, dy * p.inv_rho0, dz * p.inv_rho0);
}

// Delta of particle i: the single-gather form when the step's masses all have one bit pattern
// (mass_bits = {0 when they do, that pattern}, from k_gather), else the general one.
template <bool EXACT>
__device__ __forceinline__ float3 delta_of(const StepParams& p, int i, float4 xi,
                                           const float4* __restrict__ ps_in,
                                           const float* __restrict__ lam,
                                           const float4* __restrict__ psl,
                                           const uint32_t* __restrict__ mass_bits,
                                           const uint4* __restrict__ nbr4, int c) {
    if (__ldg(mass_bits) == 0u)
        return position_delta_uniform<EXACT>(p, p.n, psl[i], psl, __uint_as_float(__ldg(mass_bits + 1)),
                                             nbr4 + i, c);
    return position_delta<EXACT>(p, p.n, xi, lam[i], ps_in, lam, nbr4 + i, c);
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
__global__ void __launch_bounds__(kMaxPairBlock)
    k_delta_correct(const StepParams* __restrict__ P, const float4* __restrict__ ps_in,
                    const float* __restrict__ lam, const uint4* __restrict__ nbr4,
                    const uint32_t* __restrict__ cnt, float4* __restrict__ ps_out,
                    float4* __restrict__ dp4, const float4* __restrict__ psl,
                    const uint32_t* __restrict__ mass_bits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P->n) return;
    const StepParams& p = params_for(P, i);
    if (i >= p.n) return;
    const float4 xi = ps_in[i];
    const float3 d = delta_of<EXACT>(p, i, xi, ps_in, lam, psl, mass_bits, nbr4, (int)cnt[i]);
    dp4[i] = make_float4(d.x, d.y, d.z, 0.f);
    float nx = clamp_axis(xi.x + d.x, p.box_min[0], p.box_max[0]);
    float ny = clamp_axis(xi.y + d.y, p.box_min[1], p.box_max[1]);
    float nz = clamp_axis(xi.z + d.z, p.box_min[2], p.box_max[2]);
    sdf_correct(p, nx, ny, nz);
    ps_out[i] = make_float4(nx, ny, nz, xi.w);
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
// go straight to the update and the carried density/lambda/delta move into the state.  Also moves
// the gathered colour, size and reference rank into the state arrays.
template <bool EXACT>
__global__ void __launch_bounds__(kMaxPairBlock)
    k_delta_final(const StepParams* __restrict__ P, const float4* __restrict__ ps_in,
                  const float* __restrict__ lam, const uint4* __restrict__ nbr4,
                  const uint32_t* __restrict__ cnt, const float4* __restrict__ x_old,
                  float4* __restrict__ x4, float4* __restrict__ v4, float4* __restrict__ vstar4,
                  float4* __restrict__ dp4, const float4* __restrict__ col4g,
                  const float* __restrict__ sizeg, float4* __restrict__ col4,
                  float* __restrict__ size, const uint32_t* __restrict__ rref_new,
                  uint32_t* __restrict__ rref, const float* __restrict__ rho_c,
                  const float* __restrict__ lam_c, const float4* __restrict__ dp_c,
                  float* __restrict__ rho, float* __restrict__ lam_out, int has_delta,
                  const float4* __restrict__ psl, const uint32_t* __restrict__ mass_bits,
                  float4* __restrict__ xv8) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P->n) return;
    const StepParams& p = params_for(P, i);
    if (i >= p.n) return;
    const float4 xi = ps_in[i];
    float nx = xi.x, ny = xi.y, nz = xi.z;
    if (has_delta) {
        const float3 d = delta_of<EXACT>(p, i, xi, ps_in, lam, psl, mass_bits, nbr4, (int)cnt[i]);
        dp4[i] = make_float4(d.x, d.y, d.z, 0.f);
        nx = clamp_axis(xi.x + d.x, p.box_min[0], p.box_max[0]);
        ny = clamp_axis(xi.y + d.y, p.box_min[1], p.box_max[1]);
        nz = clamp_axis(xi.z + d.z, p.box_min[2], p.box_max[2]);
        sdf_correct(p, nx, ny, nz);
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
    // the same damping against each obstacle, along its SDF gradient (plain dot products)
    for (int k = 0; k < p.num_shapes; ++k) {
        float g[3];
        const float dist = sdf_eval(p.shapes[k], nx, ny, nz, g);
        const float appr = vx * g[0] + vy * g[1] + vz * g[2];
        if (dist < p.sdf_min_dist) {
            const float vnx = appr * g[0], vny = appr * g[1], vnz = appr * g[2];
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
    const float4 xn = make_float4(nx, ny, nz, xi.w), vn = make_float4(vx, vy, vz, 0.f);
    x4[i] = xn;
    v4[i] = vn;
    xv8[2 * (size_t)i] = xn;  // (x, m | v) for vorticity's single gather
    xv8[2 * (size_t)i + 1] = vn;
    col4[i] = col4g[i];
    size[i] = sizeg[i];
    rref[i] = rref_new[i];
}

// omega_i = sum_j -m_j (v_j - v_i) x grad W(x_i - x_j)  (IntegrationCUDA.cu:104-128).
// om4.w = |omega_i| for the confinement pass.
template <bool EXACT>
__global__ void __launch_bounds__(kMaxPairBlock)
    k_vorticity(const StepParams* __restrict__ P, const float4* __restrict__ x4,
                const float4* __restrict__ v4, const float4* __restrict__ xv8,
                const uint4* __restrict__ nbr4, const uint32_t* __restrict__ cnt,
                float4* __restrict__ om4, float4* __restrict__ xw4) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P->n) return;
    const StepParams& p = params_for(P, i);
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = x4[i], vi = v4[i];
    float wx = 0.f, wy = 0.f, wz = 0.f;
    for_each_pair(nbr4 + i, n, (int)cnt[i], [&](uint32_t j0, uint32_t j1, bool two) {
        const Rec8 ra = ld_rec8(xv8, j0), rb = ld_rec8(xv8, j1);
        const float4 a = ra.x, b = rb.x, va = ra.v, vb = rb.v;
        const float2 sx = sub2(f2(xi.x), make_float2(a.x, b.x));
        const float2 sy = sub2(f2(xi.y), make_float2(a.y, b.y));
        const float2 sz = sub2(f2(xi.z), make_float2(a.z, b.z));
        float2 gx, gy, gz;
        spiky2<EXACT>(p, sx, sy, sz, len2_2(sx, sy, sz), gx, gy, gz);
        const float2 ux = sub2(make_float2(va.x, vb.x), f2(vi.x));
        const float2 uy = sub2(make_float2(va.y, vb.y), f2(vi.y));
        const float2 uz = sub2(make_float2(va.z, vb.z), f2(vi.z));
        // cross(u, g) contracted as fma(u.y, g.z, -(u.z * g.y)), ...
        const float2 cx = fma2(uy, gz, mul2(f2(-1.0f), mul2(uz, gy)));
        const float2 cy = fma2(uz, gx, mul2(f2(-1.0f), mul2(ux, gz)));
        const float2 cz = fma2(ux, gy, mul2(f2(-1.0f), mul2(uy, gx)));
        wx = __fmaf_rn(-a.w, cx.x, wx);
        wy = __fmaf_rn(-a.w, cy.x, wy);
        wz = __fmaf_rn(-a.w, cz.x, wz);
        if (two) {
            wx = __fmaf_rn(-b.w, cx.y, wx);
            wy = __fmaf_rn(-b.w, cy.y, wy);
            wz = __fmaf_rn(-b.w, cz.y, wz);
        }
    });
    const float wn = __fsqrt_rn(len2(wx, wy, wz));
    om4[i] = make_float4(wx, wy, wz, wn);
    xw4[i] = make_float4(xi.x, xi.y, xi.z, wn);  // (x, |omega|) for confinement's single gather
}

// Vorticity confinement (IntegrationCUDA.cu:130-165); writes the confined velocity to the
// particle records (x, m_i / rho_i | v) for the XSPH pass.
// Capped at 48 registers (five 256-thread blocks per SM): 80 µs against 84 at 60 registers on the
// 1M scene, although 36 bytes spill; the same cap slowed vorticity and the last delta pass.
template <bool EXACT>
__global__ void __launch_bounds__(kMaxPairBlock, 5)
    k_confine(const StepParams* __restrict__ P, const float4* __restrict__ x4,
              const float4* __restrict__ v4, const float4* __restrict__ om4,
              const float* __restrict__ rho, const uint4* __restrict__ nbr4,
              const uint32_t* __restrict__ cnt, float4* __restrict__ xv8,
              const float4* __restrict__ xw4, const uint32_t* __restrict__ mass_bits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P->n) return;
    const StepParams& p = params_for(P, i);
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = x4[i], vi = v4[i], wi = om4[i];
    const float rho_i = rho[i];
    float ex = 0.f, ey = 0.f, ez = 0.f;
    // pair term m_j (|omega_i| - |omega_j|) grad W, given positions, masses and |omega_j|
    auto term = [&](float4 a, float4 b, float2 mj, float2 wj, bool two) {
        const float2 sx = sub2(f2(xi.x), make_float2(a.x, b.x));
        const float2 sy = sub2(f2(xi.y), make_float2(a.y, b.y));
        const float2 sz = sub2(f2(xi.z), make_float2(a.z, b.z));
        float2 gx, gy, gz;
        spiky2<EXACT>(p, sx, sy, sz, len2_2(sx, sy, sz), gx, gy, gz);
        const float2 s = mul2(mj, sub2(f2(wi.w), wj));
        ex = __fmaf_rn(s.x, gx.x, ex);
        ey = __fmaf_rn(s.x, gy.x, ey);
        ez = __fmaf_rn(s.x, gz.x, ez);
        if (two) {
            ex = __fmaf_rn(s.y, gx.y, ex);
            ey = __fmaf_rn(s.y, gy.y, ey);
            ez = __fmaf_rn(s.y, gz.y, ez);
        }
    };
    if (__ldg(mass_bits) == 0u) {  // one mass: (x, |omega|) in one gather, the same products
        const float m = __uint_as_float(__ldg(mass_bits + 1));
        for_each_pair(nbr4 + i, n, (int)cnt[i], [&](uint32_t j0, uint32_t j1, bool two) {
            const float4 a = __ldg(xw4 + j0), b = __ldg(xw4 + j1);
            term(a, b, f2(m), make_float2(a.w, b.w), two);
        });
    } else {
        for_each_pair(nbr4 + i, n, (int)cnt[i], [&](uint32_t j0, uint32_t j1, bool two) {
            const float4 a = __ldg(x4 + j0), b = __ldg(x4 + j1);
            term(a, b, make_float2(a.w, b.w),
                 make_float2(__ldg(&om4[j0].w), __ldg(&om4[j1].w)), two);
        });
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
    // (x, m_i / rho_i | confined v) for XSPH's single gather; vorticity, the only other reader of
    // these records, has finished, and no thread here reads another particle's record
    xv8[2 * (size_t)i] = make_float4(xi.x, xi.y, xi.z, __fdiv_rn(xi.w, rho_i));
    xv8[2 * (size_t)i + 1] = make_float4(vx, vy, vz, 0.f);
}

// XSPH viscosity (IntegrationCUDA.cu:167-195) from the confined-velocity snapshot in the records
// (x, m / rho | v).  Also leaves the bucket table all-empty for the next step.
__global__ void __launch_bounds__(kMaxPairBlock)
    k_xsph(const StepParams* __restrict__ P, const float4* __restrict__ xv8,
           const uint4* __restrict__ nbr4, const uint32_t* __restrict__ cnt,
           float4* __restrict__ v4, const uint32_t* __restrict__ kr, uint2* __restrict__ table) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P->n) return;
    {  // the walk is done: empty this step's bucket entries (thread i: the bucket starting at rank i)
        const uint32_t k = kr[i];
        if (i == 0 || kr[i - 1] != k) table[k] = make_uint2(0u, 0u);
    }
    const StepParams& p = params_for(P, i);
    const int n = p.n;
    if (i >= n) return;
    const Rec8 ri = ld_rec8(xv8, (uint32_t)i);
    const float4 xi = ri.x, vi = ri.v;
    float ax = 0.f, ay = 0.f, az = 0.f;
    for_each_pair(nbr4 + i, n, (int)cnt[i], [&](uint32_t j0, uint32_t j1, bool two) {
        const Rec8 ra = ld_rec8(xv8, j0), rb = ld_rec8(xv8, j1);
        const float4 a = ra.x, b = rb.x, va = ra.v, vb = rb.v;
        const float2 sx = sub2(f2(xi.x), make_float2(a.x, b.x));
        const float2 sy = sub2(f2(xi.y), make_float2(a.y, b.y));
        const float2 sz = sub2(f2(xi.z), make_float2(a.z, b.z));
        const float2 w = poly6_2(p, len2_2(sx, sy, sz));
        const float2 s = make_float2(a.w, b.w);  // m_j / rho_j
        const float2 tx = mul2(s, sub2(make_float2(va.x, vb.x), f2(vi.x)));
        const float2 ty = mul2(s, sub2(make_float2(va.y, vb.y), f2(vi.y)));
        const float2 tz = mul2(s, sub2(make_float2(va.z, vb.z), f2(vi.z)));
        ax = __fmaf_rn(tx.x, w.x, ax);
        ay = __fmaf_rn(ty.x, w.x, ay);
        az = __fmaf_rn(tz.x, w.x, az);
        if (two) {
            ax = __fmaf_rn(tx.y, w.y, ax);
            ay = __fmaf_rn(ty.y, w.y, ay);
            az = __fmaf_rn(tz.y, w.y, az);
        }
    });
    v4[i] = make_float4(__fmaf_rn(p.visc, ax, vi.x), __fmaf_rn(p.visc, ay, vi.y),
                        __fmaf_rn(p.visc, az, vi.z), 0.f);
}

}  // namespace akua
