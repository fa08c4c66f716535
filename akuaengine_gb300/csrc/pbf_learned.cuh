// Learned warm start of the Jacobi loop: per-particle features for the lambda network, and the
// density-constraint error that measures a step (plain or warm-started).
//
// The warm start replaces iteration 1's lambda (the one-step Jacobi estimate) by the network's
// prediction of the lambda a 20-iteration solve accumulates over the step (the sum of its
// iterations' lambdas, which is what drives the total position correction since delta-p is linear
// in lambda), blended with iteration 1's lambda by a calibrated factor.  Later iterations run the
// reference's update unchanged, so the plain iterated solver still corrects whatever the
// prediction leaves.
//
// Features of particle i at the start of the step, all by-products of iteration 1's density and
// lambda over the step's neighbour list (the walk writes them; no extra neighbour pass):
//   0 C_i = rho_i / rho0 - 1              4 the previous step's accumulated lambda
//   1 neighbour count / 32                5 |grad_i C_i| (large at the free surface)
//   2 S_i = sum_j |grad_j C_i|^2 + |grad_i C_i|^2 (the lambda denominator without epsilon)
//   3 lambda_i of iteration 1             6 grad_i C_i along gravity (which side is open)
//                                         7 |predicted velocity|
// All of them are functions of the state the step starts from, the same in plain and in
// warm-started runs (the record's own `lambda` field is not: it holds the last iteration's value).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "pbf_device.cuh"

namespace akua {

constexpr int kFeatures = 8;

// `acc`: iteration 1's density/lambda accumulator of particle i (rho, sum of |grad_j C_i|^2 and
// sum_j m_j grad W_ij in gx, gy, gz).
template <class Acc>
__device__ __forceinline__ void write_features(const StepParams& p, const Acc& acc, float lam0,
                                               int count, float lprev, float speed, float* out) {
    const float ax = acc.gx * p.inv_rho0, ay = acc.gy * p.inv_rho0, az = acc.gz * p.inv_rho0;
    const float a2 = ax * ax + ay * ay + az * az;
    const float g2 = p.gravity[0] * p.gravity[0] + p.gravity[1] * p.gravity[1] +
                     p.gravity[2] * p.gravity[2];
    const float ig = g2 > 0.f ? rsqrtf(g2) : 0.f;
    const float along = (ax * p.gravity[0] + ay * p.gravity[1] + az * p.gravity[2]) * ig;
    float4* o = reinterpret_cast<float4*>(out);
    o[0] = make_float4(acc.rho * p.inv_rho0 - 1.0f, (float)count * (1.0f / 32.0f), acc.sum + a2,
                       lam0);
    o[1] = make_float4(lprev, sqrtf(a2), along, speed);
}

// Density-constraint error at the positions a step ended with, over that step's lists:
// max_i max(rho_i / rho0 - 1, 0) (as float bits, atomically maxed) and sum_i |rho_i / rho0 - 1|.
__global__ void __launch_bounds__(128)
    k_density_error(const StepParams* __restrict__ P, const float4* __restrict__ x4,
                    const uint4* __restrict__ nbr4, const uint32_t* __restrict__ cnt,
                    uint32_t* __restrict__ max_bits, double* __restrict__ sum_abs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = P->n;
    float e = 0.f, m = 0.f;
    if (i < n) {
        const StepParams& p = params_for(P, i);
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
