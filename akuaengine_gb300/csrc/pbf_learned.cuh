// Learned warm start of the Jacobi loop: per-particle features for the lambda network, and the
// density-constraint error that judges a step (plain or warm-started).
//
// The warm start replaces iteration 1's lambda (the one-step Jacobi estimate) by the network's
// prediction of the lambda a 20-iteration solve accumulates over the step (the sum of its
// iterations' lambdas, which is what drives the total position correction since delta-p is linear
// in lambda).  Later iterations run the reference's update unchanged, so the plain iterated solver
// still corrects whatever the prediction leaves.
//
// Features of particle i at the start of the step (predicted positions x*, predicted velocity v*,
// the step's neighbour lists):
//   0 C_i = rho_i / rho0 - 1              4 the previous step's accumulated lambda
//   1 neighbour count / 32                5 mean C_j over the neighbours
//   2 S_i = sum_j |grad_j C_i|^2 + |grad_i C_i|^2 (the lambda denominator without epsilon)
//   3 lambda_i of iteration 1             6 SPH divergence of v*: sum_j m_j / rho_j (v_j - v_i) . grad W_ij
//                                         7 |v*_i|
// All of them are functions of the state the step starts from, the same in plain and in
// warm-started runs (the record's own `lambda` field is not: it holds the last iteration's value).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pbf_device.cuh"
#include "pbf_pairs.cuh"

namespace akua {

constexpr int kFeatures = 8;

// Spiky gradient dW/dx at separation d (|d|^2 = r2 < h2, r2 > 0), float math.
__device__ __forceinline__ float3 spiky_grad_fast(const StepParams& p, float dx, float dy, float dz,
                                                  float r2) {
    const float inv_r = rsqrtf(r2);
    const float r = r2 * inv_r;
    const float q = p.h - r;
    const float c = p.ks * q * q * inv_r;
    return make_float3(c * dx, c * dy, c * dz);
}

__global__ void __launch_bounds__(128)
    k_features(const StepParams* __restrict__ P, const float4* __restrict__ ps,
               const float4* __restrict__ vs, const float* __restrict__ lam0,
               const float* __restrict__ lprev, const uint4* __restrict__ nbr4,
               const uint32_t* __restrict__ cnt, float* __restrict__ feat) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = p.n;
    if (i >= n) return;
    const float4 xi = ps[i];
    const float4 vi = vs[i];  // .w = density
    const int c = (int)cnt[i];
    float gx = 0.f, gy = 0.f, gz = 0.f, s2 = 0.f, csum = 0.f, div = 0.f;
    auto pair = [&](uint32_t j) {
        const float4 a = __ldg(ps + j);
        const float4 b = __ldg(vs + j);
        const float dx = xi.x - a.x, dy = xi.y - a.y, dz = xi.z - a.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        csum += b.w * p.inv_rho0 - 1.0f;
        if (r2 > 0.f && r2 < p.h2) {
            const float3 g = spiky_grad_fast(p, dx, dy, dz, r2);
            gx += a.w * g.x;
            gy += a.w * g.y;
            gz += a.w * g.z;
            const float s = a.w * p.inv_rho0;
            s2 += s * s * (g.x * g.x + g.y * g.y + g.z * g.z);
            div += (a.w / b.w) * ((b.x - vi.x) * g.x + (b.y - vi.y) * g.y + (b.z - vi.z) * g.z);
        }
    };
    const uint4* row = nbr4 + i;
    for (int g = 0; 4 * g < c; ++g) {
        const uint4 e = row[(size_t)g * n];
        const int left = c - 4 * g;
        pair(e.x);
        if (left > 1) pair(e.y);
        if (left > 2) pair(e.z);
        if (left > 3) pair(e.w);
    }
    const float ax = gx * p.inv_rho0, ay = gy * p.inv_rho0, az = gz * p.inv_rho0;
    float4* out = reinterpret_cast<float4*>(feat) + 2 * (size_t)i;
    out[0] = make_float4(vi.w * p.inv_rho0 - 1.0f, (float)c * (1.0f / 32.0f),
                         s2 + ax * ax + ay * ay + az * az, lam0[i]);
    out[1] = make_float4(lprev[i], c > 0 ? csum / (float)c : 0.f, div,
                         sqrtf(vi.x * vi.x + vi.y * vi.y + vi.z * vi.z));
}

// Density-constraint error at the positions a step ended with, over that step's lists:
// max_i max(rho_i / rho0 - 1, 0) (as float bits, atomically maxed) and sum_i |rho_i / rho0 - 1|.
__global__ void __launch_bounds__(128)
    k_density_error(const StepParams* __restrict__ P, const float4* __restrict__ x4,
                    const uint4* __restrict__ nbr4, const uint32_t* __restrict__ cnt,
                    uint32_t* __restrict__ max_bits, double* __restrict__ sum_abs) {
    const StepParams& p = *P;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = p.n;
    float e = 0.f, m = 0.f;
    if (i < n) {
        const float4 xi = x4[i];
        float rho = xi.w * p.w0;
        const int c = (int)cnt[i];
        const uint4* row = nbr4 + i;
        for (int g = 0; 4 * g < c; ++g) {
            const uint4 t = row[(size_t)g * n];
            const uint32_t js[4] = {t.x, t.y, t.z, t.w};
            const int k_end = min(4, c - 4 * g);
            for (int k = 0; k < k_end; ++k) {
                const float4 a = __ldg(x4 + js[k]);
                const float dx = xi.x - a.x, dy = xi.y - a.y, dz = xi.z - a.z;
                rho += a.w * poly6(p, dx * dx + dy * dy + dz * dz);
            }
        }
        const float cval = rho * p.inv_rho0 - 1.0f;
        e = fabsf(cval);
        m = fmaxf(cval, 0.f);
    }
    double se = e;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        se += __shfl_xor_sync(0xffffffffu, se, o);
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sum_abs, se);
        atomicMax(max_bits, __float_as_uint(m));
    }
}

}  // namespace akua
