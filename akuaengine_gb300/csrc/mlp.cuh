// Learned lambda warm start: an 8 -> 64 -> 64 -> 64 -> 1 MLP with SiLU, BF16 weights and
// activations on the tensor cores (tcgen05, FP32 accumulation in tensor memory), trained on the
// GPU by its own forward and backward kernels.
//
// Parameters are an FP32 master copy, flattened (offsets below); kernels round W1..W3 to BF16 when
// they stage them in shared memory.  Biases, the output layer (w4, b4) and all element-wise math
// stay FP32.  Rounding points (what the host restatement reproduces):
//   x  = bf16((f - mean) * inv_std)
//   a1 = bf16(silu(x W1^T + b1)),  a2 = bf16(silu(a1 W2^T + b2)),  a3 = silu(a2 W3^T + b3)
//   y  = a3 . w4 + b4,  output = y * out_scale
// Backward of L = (1/n) sum (y - t / out_scale)^2:
//   dy = 2 (y - t') / n;  dz3 = bf16(dy w4 silu'(z3));  dz2 = bf16((dz3 W3) silu'(z2));
//   dz1 = bf16((dz2 W2) silu'(z1));  dW_l = dz_l^T a_{l-1};  db_l = sum dz_l;  dw4 = sum dy a3
//
// One CTA of 128 threads per tile of 128 samples (thread t owns sample row t, TMEM lane t).  The
// forward kernel keeps one 64-column accumulator; the gradient kernel keeps z1..z3, the input
// gradient and the three weight-gradient accumulators in tensor memory (432 of 512 columns) and
// accumulates the weight gradients over all tiles it processes before one atomic flush.
// Weight gradients are MMAs over the batch: dW^T-shaped D[out][in] = A[out][b] B[in][b] with
// A = dz^T (64 rows, padded to M = 128 with zeros) and B = a^T plus one row of ones, whose column
// of D is the bias gradient.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "tc05.cuh"

namespace akua::mlp {

constexpr int kIn = 8;
constexpr int kInPad = 16;
constexpr int kHid = 64;
constexpr int kTile = 128;
constexpr int kThreads = 128;

// FP32 parameter offsets.
constexpr int kW1 = 0;                  // [64][8]
constexpr int kB1 = kW1 + kHid * kIn;   // [64]
constexpr int kW2 = kB1 + kHid;         // [64][64]
constexpr int kB2 = kW2 + kHid * kHid;  // [64]
constexpr int kW3 = kB2 + kHid;         // [64][64]
constexpr int kB3 = kW3 + kHid * kHid;  // [64]
constexpr int kW4 = kB3 + kHid;         // [64]
constexpr int kB4 = kW4 + kHid;         // [1]
constexpr int kParams = kB4 + 1;        // 8961
// Normalisation: mean[8], inv_std[8], out_scale, blend (see k_mlp_forward).
constexpr int kNorm = 2 * kIn + 2;
constexpr int kLam0 = 3;  // input feature holding iteration 1's lambda

constexpr int kErrTimeout = 1;

// sigmoid(z) = (1 + tanh(z / 2)) / 2 through the hardware tanh approximation (PTX tanh.approx,
// relative error about 2^-11); training and inference use the same forms.
__device__ __forceinline__ float tanh_hw(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sigmoid(float z) { return __fmaf_rn(0.5f, tanh_hw(0.5f * z), 0.5f); }
__device__ __forceinline__ float silu(float z) { return z * sigmoid(z); }
// Inference: silu of two values, the tanh evaluated on an FP16 pair (tanh.approx.f16x2: one
// multi-function operation for two activations; its error, about 2^-11 relative, is below the
// BF16 rounding the hidden activations get next).
__device__ __forceinline__ float2 silu2(float z0, float z1) {
    const __half2 hz = __floats2half2_rn(0.5f * z0, 0.5f * z1);
    uint32_t in, out;
    memcpy(&in, &hz, 4);
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(out) : "r"(in));
    __half2 ht;
    memcpy(&ht, &out, 4);
    const float2 t = __half22float2(ht);
    return make_float2(z0 * __fmaf_rn(0.5f, t.x, 0.5f), z1 * __fmaf_rn(0.5f, t.y, 0.5f));
}
__device__ __forceinline__ float dsilu(float z) {
    const float s = sigmoid(z);
    return s * (1.0f + z * (1.0f - s));
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ uint16_t bf16_bits(float a) {
    const __nv_bfloat16 v = __float2bfloat16_rn(a);
    return *reinterpret_cast<const uint16_t*>(&v);
}
__device__ __forceinline__ float bf16_round(float a) {
    return __bfloat162float(__float2bfloat16_rn(a));
}

// Row `row` of a K-major tile with K = 64: 64 values as eight 16-byte core-matrix rows.
__device__ __forceinline__ void store_row64(uint8_t* tile, int row, const float* v, int c0) {
    // v holds 16 values for columns c0 .. c0+15
    *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(row, c0, 64)) =
        make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]),
                   pack_bf16(v[6], v[7]));
    *reinterpret_cast<uint4*>(tile + tc::kmajor_offset(row, c0 + 8, 64)) =
        make_uint4(pack_bf16(v[8], v[9]), pack_bf16(v[10], v[11]), pack_bf16(v[12], v[13]),
                   pack_bf16(v[14], v[15]));
}

// Column `col` of a transposed K-major tile with K = 128 (rows = features, k = sample): 16 values
// for feature rows r0 .. r0+15 of sample `col`.
__device__ __forceinline__ void store_col128(uint8_t* tile, int col, const float* v, int r0) {
#pragma unroll
    for (int q = 0; q < 16; ++q)
        *reinterpret_cast<uint16_t*>(tile + tc::kmajor_offset(r0 + q, col, 128)) = bf16_bits(v[q]);
}

// Stages a [64][K] weight (row-major FP32 [64][kin]) as a BF16 K-major B operand with K = kpad
// columns (zeros beyond kin); `transposed` stages W^T ([in][out]) instead.
__device__ __forceinline__ void stage_weight(uint8_t* dst, const float* __restrict__ w, int kin,
                                             int kpad, bool transposed, int t) {
    for (int e = t; e < kHid * kpad; e += kThreads) {
        const int r = e / kpad, k = e - r * kpad;  // operand row r, column k
        float v = 0.f;
        if (!transposed) {
            if (k < kin) v = w[r * kin + k];  // B[out][in] = W[out][in]
        } else {
            v = w[k * kin + r];  // B[in][out] = W[out][in]; kin == kpad == 64
        }
        *reinterpret_cast<uint16_t*>(dst + tc::kmajor_offset(r, k, kpad)) = bf16_bits(v);
    }
}

// BF16 operand images of W1, W2, W3 in the forward pass's shared-memory layout, rebuilt by
// k_mlp_image whenever the parameters change; a forward CTA copies them instead of converting.
constexpr int kImageBytes = (kHid * kInPad + 2 * kHid * kHid) * 2;

__global__ void __launch_bounds__(kThreads)
    k_mlp_image(const float* __restrict__ params, uint8_t* __restrict__ image) {
    const int t = threadIdx.x;
    stage_weight(image, params + kW1, kIn, kInPad, false, t);
    stage_weight(image + kHid * kInPad * 2, params + kW2, kHid, kHid, false, t);
    stage_weight(image + kHid * kInPad * 2 + kHid * kHid * 2, params + kW3, kHid, kHid, false, t);
}

// ------------------------------------------------------------------------------------ forward
struct FwdSmem {
    alignas(128) uint8_t w1[kHid * kInPad * 2];
    alignas(128) uint8_t w2[kHid * kHid * 2];
    alignas(128) uint8_t w3[kHid * kHid * 2];
    alignas(128) uint8_t x[kTile * kInPad * 2];
    alignas(128) uint8_t h[kTile * kHid * 2];
    float b1[kHid], b2[kHid], b3[kHid], w4[kHid];
    float norm[kNorm];
    float b4;
    alignas(8) uint64_t bar;
    uint32_t tmem;
};

// Epilogue of a hidden layer: TMEM columns [col, col+64) of this thread's row -> bias, SiLU,
// BF16 -> row t of the next layer's A tile.
__device__ __forceinline__ void hidden_epilogue(uint32_t taddr, const float* b, uint8_t* h, int t) {
    uint32_t r[4][16];
#pragma unroll
    for (int c = 0; c < 4; ++c) tc::tmem_ld16_async(taddr + 16 * c, r[c]);
    tc::tmem_wait_ld();
#pragma unroll
    for (int c = 0; c < 4; ++c) tc::tmem_after_wait(r[c]);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        float v[16];
#pragma unroll
        for (int q = 0; q < 16; q += 2) {
            const float2 a = silu2(__uint_as_float(r[c][q]) + b[16 * c + q],
                                   __uint_as_float(r[c][q + 1]) + b[16 * c + q + 1]);
            v[q] = a.x;
            v[q + 1] = a.y;
        }
        store_row64(h, t, v, 16 * c);
    }
}

// Output layer on the FP32 pipe: b4 + sum_c w4[c] silu(z3[c] + b3[c]).
__device__ __forceinline__ float output_layer(uint32_t taddr, const float* b3, const float* w4,
                                              float b4) {
    uint32_t r[4][16];
#pragma unroll
    for (int c = 0; c < 4; ++c) tc::tmem_ld16_async(taddr + 16 * c, r[c]);
    tc::tmem_wait_ld();
#pragma unroll
    for (int c = 0; c < 4; ++c) tc::tmem_after_wait(r[c]);
    float y = b4;
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int q = 0; q < 16; q += 2) {
            const float2 a = silu2(__uint_as_float(r[c][q]) + b3[16 * c + q],
                                   __uint_as_float(r[c][q + 1]) + b3[16 * c + q + 1]);
            y = __fmaf_rn(w4[16 * c + q], a.x, y);
            y = __fmaf_rn(w4[16 * c + q + 1], a.y, y);
        }
    return y;
}

__device__ __forceinline__ void load_features(const float* __restrict__ feat, int i, int n,
                                              const float* norm, float (&f)[kIn]) {
    if (i < n) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(feat) + 2 * (size_t)i);
        const float4 b = __ldg(reinterpret_cast<const float4*>(feat) + 2 * (size_t)i + 1);
        f[0] = a.x; f[1] = a.y; f[2] = a.z; f[3] = a.w;
        f[4] = b.x; f[5] = b.y; f[6] = b.z; f[7] = b.w;
    } else {
#pragma unroll
        for (int k = 0; k < kIn; ++k) f[k] = norm[k];
    }
}

// Features (n x 8, FP32) -> out2[i] = the network's estimate p_i (output * out_scale) and
// out[i] = lambda0_i + blend * (p_i - lambda0_i), lambda0 = feature 3 (blend 1: out = p); the
// latter also into out4[4 i] when given.
__global__ void __launch_bounds__(kThreads)
    k_mlp_forward(const float* __restrict__ params, const uint8_t* __restrict__ image,
                  const float* __restrict__ norm, const float* __restrict__ feat, int n,
                  float* __restrict__ out, float* __restrict__ out2, float* __restrict__ out4,
                  uint32_t* __restrict__ err) {
    __shared__ FwdSmem S;
    static_assert(offsetof(FwdSmem, w2) == offsetof(FwdSmem, w1) + sizeof(S.w1) &&
                      offsetof(FwdSmem, w3) == offsetof(FwdSmem, w2) + sizeof(S.w2) &&
                      sizeof(S.w1) + sizeof(S.w2) + sizeof(S.w3) == kImageBytes,
                  "the weight image is w1, w2, w3 back to back");
    const int t = threadIdx.x, warp = t >> 5;
    {
        const uint4* src = reinterpret_cast<const uint4*>(image);
        uint4* dst = reinterpret_cast<uint4*>(S.w1);
        for (int k = t; k < kImageBytes / 16; k += kThreads) dst[k] = __ldg(src + k);
    }
    if (t < kHid) {
        S.b1[t] = params[kB1 + t];
        S.b2[t] = params[kB2 + t];
        S.b3[t] = params[kB3 + t];
        S.w4[t] = params[kW4 + t];
    }
    if (t < kNorm) S.norm[t] = norm[t];
    if (t == 0) {
        S.b4 = params[kB4];
        tc::mbar_init(&S.bar, 1);
    }
    // columns 8..15 of the input tile stay zero
    *reinterpret_cast<uint4*>(S.x + tc::kmajor_offset(t, 8, kInPad)) = make_uint4(0, 0, 0, 0);
    if (warp == 0) tc::tmem_alloc(&S.tmem, 64);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = S.tmem;
    const uint32_t lane = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t idesc = tc::idesc_bf16(128, 64);
    const uint64_t dx = tc::smem_desc(tc::smem_addr(S.x), 128, kInPad * 16);
    const uint64_t dw1 = tc::smem_desc(tc::smem_addr(S.w1), 128, kInPad * 16);
    const uint32_t sh = tc::smem_addr(S.h), sw2 = tc::smem_addr(S.w2), sw3 = tc::smem_addr(S.w3);
    uint32_t phase = 0;
    bool ok = true;
    const int tiles = (n + kTile - 1) / kTile;
    float fnext[kIn];
    load_features(feat, blockIdx.x * kTile + t, n, S.norm, fnext);
    const float blend = S.norm[2 * kIn + 1];
    for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int i = tile * kTile + t;
        const float lam0 = fnext[kLam0];
        float f[kIn];
#pragma unroll
        for (int k = 0; k < kIn; ++k) f[k] = (fnext[k] - S.norm[k]) * S.norm[kIn + k];
        if (tile + (int)gridDim.x < tiles)  // the next tile's features, in flight meanwhile
            load_features(feat, (tile + gridDim.x) * kTile + t, n, S.norm, fnext);
        *reinterpret_cast<uint4*>(S.x + tc::kmajor_offset(t, 0, kInPad)) =
            make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]),
                       pack_bf16(f[6], f[7]));
        // layer 1
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        if (t == 0) {
            tc::fence_after_sync();
            tc::mma_bf16(tmem, dx, dw1, idesc, 0);
            tc::mma_commit(&S.bar);
        }
        ok = __syncthreads_and(tc::mbar_wait(&S.bar, phase));
        phase ^= 1;
        if (!ok) break;
        tc::fence_after_sync();
        hidden_epilogue(lane, S.b1, S.h, t);
        // layers 2 and 3
        for (int layer = 0; layer < 2 && ok; ++layer) {
            tc::fence_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            if (t == 0) {
                tc::fence_after_sync();
                const uint32_t sw = layer == 0 ? sw2 : sw3;
#pragma unroll
                for (int s = 0; s < kHid / 16; ++s)
                    tc::mma_bf16(tmem, tc::smem_desc(sh + 256 * s, 128, kHid * 16),
                                 tc::smem_desc(sw + 256 * s, 128, kHid * 16), idesc, s > 0);
                tc::mma_commit(&S.bar);
            }
            ok = __syncthreads_and(tc::mbar_wait(&S.bar, phase));
            phase ^= 1;
            if (!ok) break;
            tc::fence_after_sync();
            if (layer == 0) hidden_epilogue(lane, S.b2, S.h, t);
        }
        if (!ok) break;
        const float y = output_layer(lane, S.b3, S.w4, S.b4);
        if (i < n) {
            const float o = y * S.norm[2 * kIn];
            const float used = blend == 1.0f ? o : __fmaf_rn(blend, o - lam0, lam0);
            out[i] = used;
            if (out2) out2[i] = o;
            if (out4) out4[4 * (size_t)i] = used;  // a float4 array's 4th component
        }
        tc::fence_before_sync();
    }
    if (!ok && t == 0) atomicOr(err, (uint32_t)kErrTimeout);
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_free(tmem, 64);
    }
}

// ----------------------------------------------------------------------------------- gradient
// TMEM columns.
constexpr uint32_t kColZ1 = 0, kColZ2 = 64, kColZ3 = 128, kColDA = 192;
constexpr uint32_t kColG3 = 256, kColG2 = 336, kColG1 = 416;  // 80, 80, 16 columns
constexpr uint32_t kGradCols = 512;
constexpr int kNT = 80;  // rows of a transposed activation operand: 64 features, ones, zeros

struct GradSmem {
    alignas(128) uint8_t w1[kHid * kInPad * 2];      // B: [out][in16]
    alignas(128) uint8_t w2[kHid * kHid * 2];        // B: [out][in]
    alignas(128) uint8_t w3[kHid * kHid * 2];
    alignas(128) uint8_t w2t[kHid * kHid * 2];       // B: [in][out]
    alignas(128) uint8_t w3t[kHid * kHid * 2];
    alignas(128) uint8_t x[kTile * kInPad * 2];      // A: [b][in16]
    alignas(128) uint8_t a1[kTile * kHid * 2];       // A: [b][64]
    alignas(128) uint8_t a2[kTile * kHid * 2];
    alignas(128) uint8_t xT[kInPad * kTile * 2];     // B: [in16][b]: rows 0-7 x, row 8 ones
    alignas(128) uint8_t a1T[kNT * kTile * 2];       // B: [80][b]: rows 0-63 a1, row 64 ones
    alignas(128) uint8_t a2T[kNT * kTile * 2];
    alignas(128) uint8_t dz[kTile * kHid * 2];       // A: [b][64]
    alignas(128) uint8_t dzT[kTile * kTile * 2];     // A: [128][b]: rows 0-63 dz, rest zero
    float b1[kHid], b2[kHid], b3[kHid], w4[kHid];
    float norm[kNorm];
    float b4;
    float gw4[kHid + 1];  // dw4, db4
    float loss;
    alignas(8) uint64_t bar;
    uint32_t tmem;
};

constexpr size_t kGradSmem = sizeof(GradSmem);

// Accumulates into grad[kParams] (dL/dparams) and grad[kParams] += loss.  Targets are in output
// units (lambda); the loss is over `n_total` samples (this call may see a slice of them).
__global__ void __launch_bounds__(kThreads)
    k_mlp_grad(const float* __restrict__ params, const float* __restrict__ norm,
               const float* __restrict__ feat, const float* __restrict__ target, int n,
               float inv_n_total, float* __restrict__ grad, uint32_t* __restrict__ err) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    GradSmem& S = *reinterpret_cast<GradSmem*>(smem_raw);
    const int t = threadIdx.x, warp = t >> 5;
    stage_weight(S.w1, params + kW1, kIn, kInPad, false, t);
    stage_weight(S.w2, params + kW2, kHid, kHid, false, t);
    stage_weight(S.w3, params + kW3, kHid, kHid, false, t);
    stage_weight(S.w2t, params + kW2, kHid, kHid, true, t);
    stage_weight(S.w3t, params + kW3, kHid, kHid, true, t);
    if (t < kHid) {
        S.b1[t] = params[kB1 + t];
        S.b2[t] = params[kB2 + t];
        S.b3[t] = params[kB3 + t];
        S.w4[t] = params[kW4 + t];
    }
    if (t <= kHid) S.gw4[t] = 0.f;
    if (t < kNorm) S.norm[t] = norm[t];
    if (t == 0) {
        S.b4 = params[kB4];
        S.loss = 0.f;
        tc::mbar_init(&S.bar, 1);
    }
    // constant parts of the operand tiles: input padding, ones rows, zero rows
    {
        const uint16_t one = bf16_bits(1.0f);
        *reinterpret_cast<uint4*>(S.x + tc::kmajor_offset(t, 8, kInPad)) = make_uint4(0, 0, 0, 0);
        for (int r = kIn; r < kInPad; ++r)
            *reinterpret_cast<uint16_t*>(S.xT + tc::kmajor_offset(r, t, kTile)) =
                r == kIn ? one : (uint16_t)0;
        for (int r = kHid; r < kNT; ++r) {
            const uint16_t v = r == kHid ? one : (uint16_t)0;
            *reinterpret_cast<uint16_t*>(S.a1T + tc::kmajor_offset(r, t, kTile)) = v;
            *reinterpret_cast<uint16_t*>(S.a2T + tc::kmajor_offset(r, t, kTile)) = v;
        }
        for (int r = kHid; r < kTile; ++r)
            *reinterpret_cast<uint16_t*>(S.dzT + tc::kmajor_offset(r, t, kTile)) = 0;
    }
    if (warp == 0) tc::tmem_alloc(&S.tmem, kGradCols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = S.tmem;
    const uint32_t lane = tmem + ((uint32_t)(warp * 32) << 16);
    const uint32_t id64 = tc::idesc_bf16(128, 64);
    const uint32_t id80 = tc::idesc_bf16(128, kNT);
    const uint32_t id16 = tc::idesc_bf16(128, 16);
    const uint32_t sx = tc::smem_addr(S.x), sw1 = tc::smem_addr(S.w1);
    const uint32_t sa1 = tc::smem_addr(S.a1), sa2 = tc::smem_addr(S.a2);
    const uint32_t sw2 = tc::smem_addr(S.w2), sw3 = tc::smem_addr(S.w3);
    const uint32_t sw2t = tc::smem_addr(S.w2t), sw3t = tc::smem_addr(S.w3t);
    const uint32_t sxT = tc::smem_addr(S.xT), sa1T = tc::smem_addr(S.a1T);
    const uint32_t sa2T = tc::smem_addr(S.a2T), sdz = tc::smem_addr(S.dz);
    const uint32_t sdzT = tc::smem_addr(S.dzT);
    const float inv_scale = 1.0f / S.norm[2 * kIn];
    uint32_t phase = 0;
    uint32_t acc = 0;  // weight-gradient accumulators hold data
    bool ok = true;

    // issue helpers (thread 0 only)
    auto gemm_k64 = [&](uint32_t d, uint32_t a, uint32_t b) {  // D = A[128][64] B[64][64]^T
#pragma unroll
        for (int s = 0; s < 4; ++s)
            tc::mma_bf16(d, tc::smem_desc(a + 256 * s, 128, kHid * 16),
                         tc::smem_desc(b + 256 * s, 128, kHid * 16), id64, s > 0);
    };
    auto gemm_batch = [&](uint32_t d, uint32_t b, uint32_t idesc) {  // D += dzT[128][b] B[N][b]^T
#pragma unroll
        for (int s = 0; s < kTile / 16; ++s)
            tc::mma_bf16(d, tc::smem_desc(sdzT + 256 * s, 128, kTile * 16),
                         tc::smem_desc(b + 256 * s, 128, kTile * 16), idesc, (acc | s) != 0);
    };
    auto sync_issue = [&]() {
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
    };
    auto wait = [&]() {
        ok = __syncthreads_and(tc::mbar_wait(&S.bar, phase));
        phase ^= 1;
        tc::fence_after_sync();
        return ok;
    };

    const int tiles = (n + kTile - 1) / kTile;
    for (int tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
        const int i = tile * kTile + t;
        const bool valid = i < n;
        float f[kIn];
        if (valid) {
            const float4 a = reinterpret_cast<const float4*>(feat)[2 * (size_t)i];
            const float4 b = reinterpret_cast<const float4*>(feat)[2 * (size_t)i + 1];
            f[0] = a.x; f[1] = a.y; f[2] = a.z; f[3] = a.w;
            f[4] = b.x; f[5] = b.y; f[6] = b.z; f[7] = b.w;
        } else {
#pragma unroll
            for (int k = 0; k < kIn; ++k) f[k] = S.norm[k];
        }
#pragma unroll
        for (int k = 0; k < kIn; ++k) f[k] = (f[k] - S.norm[k]) * S.norm[kIn + k];
        *reinterpret_cast<uint4*>(S.x + tc::kmajor_offset(t, 0, kInPad)) =
            make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]),
                       pack_bf16(f[6], f[7]));
#pragma unroll
        for (int k = 0; k < kIn; ++k)
            *reinterpret_cast<uint16_t*>(S.xT + tc::kmajor_offset(k, t, kTile)) = bf16_bits(f[k]);
        const float tgt = valid ? target[i] * inv_scale : 0.f;

        // z1 = x W1^T
        sync_issue();
        if (t == 0) {
            tc::fence_after_sync();
            tc::mma_bf16(tmem + kColZ1, tc::smem_desc(sx, 128, kInPad * 16),
                         tc::smem_desc(sw1, 128, kInPad * 16), id64, 0);
            tc::mma_commit(&S.bar);
        }
        if (!wait()) break;
        // a1 -> A and B^T tiles; z2 = a1 W2^T
#pragma unroll 1
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tc::tmem_ld16(lane + kColZ1 + c0, v);
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] = silu(v[q] + S.b1[c0 + q]);
            store_row64(S.a1, t, v, c0);
            store_col128(S.a1T, t, v, c0);
        }
        sync_issue();
        if (t == 0) {
            tc::fence_after_sync();
            gemm_k64(tmem + kColZ2, sa1, sw2);
            tc::mma_commit(&S.bar);
        }
        if (!wait()) break;
#pragma unroll 1
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tc::tmem_ld16(lane + kColZ2 + c0, v);
#pragma unroll
            for (int q = 0; q < 16; ++q) v[q] = silu(v[q] + S.b2[c0 + q]);
            store_row64(S.a2, t, v, c0);
            store_col128(S.a2T, t, v, c0);
        }
        sync_issue();
        if (t == 0) {
            tc::fence_after_sync();
            gemm_k64(tmem + kColZ3, sa2, sw3);
            tc::mma_commit(&S.bar);
        }
        if (!wait()) break;
        // output, loss, dy
        float y = S.b4;
#pragma unroll 1
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16];
            tc::tmem_ld16(lane + kColZ3 + c0, v);
#pragma unroll
            for (int q = 0; q < 16; ++q) y = __fmaf_rn(S.w4[c0 + q], silu(v[q] + S.b3[c0 + q]), y);
        }
        const float e = valid ? y - tgt : 0.f;
        const float dy = 2.0f * e * inv_n_total;
        {
            float l = e * e * inv_n_total;
#pragma unroll
            for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
            if ((t & 31) == 0) atomicAdd(&S.loss, l);
        }
        // dz3 = dy w4 silu'(z3); dw4 += dy a3; db4 += dy
#pragma unroll 1
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float v[16], g[16];
            tc::tmem_ld16(lane + kColZ3 + c0, v);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const float z = v[q] + S.b3[c0 + q];
                g[q] = dy * silu(z);
                v[q] = dy * S.w4[c0 + q] * dsilu(z);
            }
            store_row64(S.dz, t, v, c0);
            store_col128(S.dzT, t, v, c0);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                float s = g[q];
#pragma unroll
                for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if ((t & 31) == 0) atomicAdd(&S.gw4[c0 + q], s);
            }
        }
        {
            float s = dy;
#pragma unroll
            for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if ((t & 31) == 0) atomicAdd(&S.gw4[kHid], s);
        }
        // da2 = dz3 W3; dW3|db3 += dz3^T [a2 | 1]
        sync_issue();
        if (t == 0) {
            tc::fence_after_sync();
            gemm_k64(tmem + kColDA, sdz, sw3t);
            gemm_batch(tmem + kColG3, sa2T, id80);
            tc::mma_commit(&S.bar);
        }
        if (!wait()) break;
        // dz2 = da2 silu'(z2)
#pragma unroll 1
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float d[16], z[16];
            tc::tmem_ld16(lane + kColDA + c0, d);
            tc::tmem_ld16(lane + kColZ2 + c0, z);
#pragma unroll
            for (int q = 0; q < 16; ++q) d[q] = d[q] * dsilu(z[q] + S.b2[c0 + q]);
            store_row64(S.dz, t, d, c0);
            store_col128(S.dzT, t, d, c0);
        }
        // da1 = dz2 W2; dW2|db2 += dz2^T [a1 | 1]
        sync_issue();
        if (t == 0) {
            tc::fence_after_sync();
            gemm_k64(tmem + kColDA, sdz, sw2t);
            gemm_batch(tmem + kColG2, sa1T, id80);
            tc::mma_commit(&S.bar);
        }
        if (!wait()) break;
        // dz1 = da1 silu'(z1); dW1|db1 += dz1^T [x | 1]
#pragma unroll 1
        for (int c0 = 0; c0 < kHid; c0 += 16) {
            float d[16], z[16];
            tc::tmem_ld16(lane + kColDA + c0, d);
            tc::tmem_ld16(lane + kColZ1 + c0, z);
#pragma unroll
            for (int q = 0; q < 16; ++q) d[q] = d[q] * dsilu(z[q] + S.b1[c0 + q]);
            store_col128(S.dzT, t, d, c0);
        }
        sync_issue();
        if (t == 0) {
            tc::fence_after_sync();
            gemm_batch(tmem + kColG1, sxT, id16);
            tc::mma_commit(&S.bar);
        }
        if (!wait()) break;
        acc = 1;
        tc::fence_before_sync();
    }
    __syncthreads();
    // flush: rows 0..63 of the weight-gradient accumulators live in warps 0 and 1
    if (ok && acc && warp < 2) {
        const int o = t;  // output feature
#pragma unroll 1
        for (int c0 = 0; c0 < kNT; c0 += 16) {
            float v[16];
            tc::tmem_ld16(lane + kColG3 + c0, v);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int c = c0 + q;
                if (c < kHid) atomicAdd(&grad[kW3 + o * kHid + c], v[q]);
                else if (c == kHid) atomicAdd(&grad[kB3 + o], v[q]);
            }
            tc::tmem_ld16(lane + kColG2 + c0, v);
#pragma unroll
            for (int q = 0; q < 16; ++q) {
                const int c = c0 + q;
                if (c < kHid) atomicAdd(&grad[kW2 + o * kHid + c], v[q]);
                else if (c == kHid) atomicAdd(&grad[kB2 + o], v[q]);
            }
        }
        float v[16];
        tc::tmem_ld16(lane + kColG1, v);
#pragma unroll
        for (int q = 0; q < kIn; ++q) atomicAdd(&grad[kW1 + o * kIn + q], v[q]);
        atomicAdd(&grad[kB1 + o], v[kIn]);
    }
    if (ok && acc) {
        if (t <= kHid) atomicAdd(&grad[kW4 + t], S.gw4[t]);
        if (t == 0) atomicAdd(&grad[kParams], S.loss);
    }
    if (!ok && t == 0) atomicOr(err, (uint32_t)kErrTimeout);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_free(tmem, kGradCols);
    }
}

// Adam on the FP32 master parameters; clears the gradient (and the loss slot) afterwards.
__global__ void k_mlp_adam(float* __restrict__ params, float* __restrict__ grad,
                           float* __restrict__ m, float* __restrict__ v, float lr, float beta1,
                           float beta2, float eps, float bc1, float bc2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > kParams) return;
    if (k == kParams) {
        grad[k] = 0.f;
        return;
    }
    const float g = grad[k];
    const float mk = beta1 * m[k] + (1.0f - beta1) * g;
    const float vk = beta2 * v[k] + (1.0f - beta2) * g * g;
    m[k] = mk;
    v[k] = vk;
    params[k] -= lr * (mk / bc1) / (sqrtf(vk / bc2) + eps);
    grad[k] = 0.f;
}

}  // namespace akua::mlp
