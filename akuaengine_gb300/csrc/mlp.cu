// C ABI of the learned-lambda network (akua_mlp_*): parameters, normalisation, the tensor-core
// forward pass, the gradient of the mean squared error and an Adam step, all on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "akua_pbf.h"
#include "mlp.cuh"
#include "mlp_handle.h"

static_assert(AKUA_MLP_PARAMS == akua::mlp::kParams, "parameter count");
static_assert(AKUA_MLP_NORM == akua::mlp::kNorm, "normalisation size");

namespace {

int status_of(cudaError_t e) {
    if (e == cudaSuccess) return AKUA_OK;
    if (e == cudaErrorMemoryAllocation) return AKUA_ERR_OUT_OF_MEMORY;
    return AKUA_ERR_CUDA;
}

struct Guard {
    int prev = -1;
    explicit Guard(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
        else prev = -1;
    }
    ~Guard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

int launch_grad(akua_mlp* m, const float* feat, const float* target, int32_t n, cudaStream_t st) {
    static bool attr_set[64] = {};
    if (m->device < 64 && !attr_set[m->device]) {
        cudaError_t e = cudaFuncSetAttribute(akua::mlp::k_mlp_grad,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)akua::mlp::kGradSmem);
        if (e != cudaSuccess) return status_of(e);
        attr_set[m->device] = true;
    }
    const int tiles = (n + akua::mlp::kTile - 1) / akua::mlp::kTile;
    const int grid = std::max(1, std::min(tiles, m->sms));  // one CTA per SM (all of TMEM)
    akua::mlp::k_mlp_grad<<<grid, akua::mlp::kThreads, akua::mlp::kGradSmem, st>>>(
        m->params, m->norm, feat, target, n, 1.0f / (float)n, m->grad, m->err);
    return status_of(cudaGetLastError());
}

}  // namespace

namespace akua::mlp {
// Used by the step (pbf_solver.cu): the forward pass writing lambda (and its running sum).
int enqueue_forward(const akua_mlp* m, const float* feat, int n, float* out, float* out2,
                    float* out4, cudaStream_t st) {
    const int tiles = (n + kTile - 1) / kTile;
    const int grid = std::max(1, std::min(tiles, 5 * m->sms));  // 5 x 40 KB of shared memory
    k_mlp_forward<<<grid, kThreads, 0, st>>>(m->params, m->image, m->norm, feat, n, out, out2,
                                             out4, m->err);
    return status_of(cudaGetLastError());
}
}  // namespace akua::mlp

extern "C" {

int akua_mlp_create(akua_mlp** out) {
    if (!out) return AKUA_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    akua_mlp* m = new (std::nothrow) akua_mlp();
    if (!m) return AKUA_ERR_OUT_OF_MEMORY;
    cudaError_t e = cudaGetDevice(&m->device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, m->device);
    const size_t pb = sizeof(float) * akua::mlp::kParams;
    if (e == cudaSuccess) e = cudaMalloc(&m->params, pb);
    if (e == cudaSuccess) e = cudaMalloc(&m->grad, pb + sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->m, pb);
    if (e == cudaSuccess) e = cudaMalloc(&m->v, pb);
    if (e == cudaSuccess) e = cudaMalloc(&m->norm, sizeof(float) * akua::mlp::kNorm);
    if (e == cudaSuccess) e = cudaMalloc(&m->err, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMalloc(&m->image, akua::mlp::kImageBytes);
    if (e == cudaSuccess) e = cudaMemset(m->image, 0, akua::mlp::kImageBytes);  // zero weights
    if (e == cudaSuccess) e = cudaMemset(m->params, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(m->grad, 0, pb + sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(m->m, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(m->v, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(m->err, 0, sizeof(uint32_t));
    if (e == cudaSuccess) {
        float norm[akua::mlp::kNorm];
        for (int k = 0; k < akua::mlp::kIn; ++k) {
            norm[k] = 0.0f;
            norm[akua::mlp::kIn + k] = 1.0f;
        }
        norm[2 * akua::mlp::kIn] = 1.0f;
        norm[2 * akua::mlp::kIn + 1] = 1.0f;
        e = cudaMemcpy(m->norm, norm, sizeof(norm), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        akua_mlp_destroy(m);
        return status_of(e);
    }
    *out = m;
    return AKUA_OK;
}

int akua_mlp_destroy(akua_mlp* m) {
    if (!m) return AKUA_ERR_INVALID_ARGUMENT;
    Guard g(m->device);
    cudaDeviceSynchronize();
    for (void* p : {(void*)m->params, (void*)m->grad, (void*)m->m, (void*)m->v, (void*)m->norm,
                    (void*)m->err, (void*)m->image})
        if (p) cudaFree(p);
    delete m;
    return AKUA_OK;
}

int akua_mlp_set_params(akua_mlp* m, const float* host, int32_t count) {
    if (!m || !host || count != akua::mlp::kParams) return AKUA_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < count; ++k)
        if (!std::isfinite(host[k])) return AKUA_ERR_INVALID_ARGUMENT;
    Guard g(m->device);
    const size_t pb = sizeof(float) * akua::mlp::kParams;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(m->params, host, pb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        akua::mlp::k_mlp_image<<<1, akua::mlp::kThreads>>>(m->params, m->image);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemset(m->m, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(m->v, 0, pb);
    if (e == cudaSuccess) e = cudaMemset(m->grad, 0, pb + sizeof(float));
    m->adam_steps = 0;
    return status_of(e);
}

int akua_mlp_get_params(akua_mlp* m, float* host, int32_t count) {
    if (!m || !host || count != akua::mlp::kParams) return AKUA_ERR_INVALID_ARGUMENT;
    Guard g(m->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy(host, m->params, sizeof(float) * count, cudaMemcpyDeviceToHost);
    return status_of(e);
}

int akua_mlp_set_normalization(akua_mlp* m, const float* host, int32_t count) {
    if (!m || !host || count != akua::mlp::kNorm) return AKUA_ERR_INVALID_ARGUMENT;
    for (int k = 0; k < count; ++k)
        if (!std::isfinite(host[k])) return AKUA_ERR_INVALID_ARGUMENT;
    if (host[2 * akua::mlp::kIn] == 0.0f) return AKUA_ERR_INVALID_ARGUMENT;
    Guard g(m->device);
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy(m->norm, host, sizeof(float) * count, cudaMemcpyHostToDevice);
    return status_of(e);
}

int akua_mlp_forward(akua_mlp* m, const float* features, float* out, int32_t n, void* stream) {
    if (!m || n < 0 || (n > 0 && (!features || !out))) return AKUA_ERR_INVALID_ARGUMENT;
    if (n == 0) return AKUA_OK;
    Guard g(m->device);
    return akua::mlp::enqueue_forward(m, features, n, out, nullptr, nullptr, (cudaStream_t)stream);
}

int akua_mlp_gradient(akua_mlp* m, const float* features, const float* targets, int32_t n,
                      float* hostGrad, float* hostLoss, void* stream) {
    if (!m || n <= 0 || !features || !targets) return AKUA_ERR_INVALID_ARGUMENT;
    Guard g(m->device);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t gb = sizeof(float) * (akua::mlp::kParams + 1);
    cudaError_t e = cudaMemsetAsync(m->grad, 0, gb, st);
    if (e != cudaSuccess) return status_of(e);
    const int rc = launch_grad(m, features, targets, n, st);
    if (rc != AKUA_OK) return rc;
    std::vector<float> tmp(akua::mlp::kParams + 1);
    e = cudaMemcpyAsync(tmp.data(), m->grad, gb, cudaMemcpyDeviceToHost, st);
    uint32_t err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err, m->err, sizeof(err), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->grad, 0, gb, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return status_of(e);
    if (err) return AKUA_ERR_DEVICE_CHECK;
    if (hostGrad) std::memcpy(hostGrad, tmp.data(), sizeof(float) * akua::mlp::kParams);
    if (hostLoss) *hostLoss = tmp[akua::mlp::kParams];
    return AKUA_OK;
}

int akua_mlp_adam_step(akua_mlp* m, const float* features, const float* targets, int32_t n,
                       float learningRate, void* stream) {
    if (!m || n <= 0 || !features || !targets || !(learningRate > 0.0f))
        return AKUA_ERR_INVALID_ARGUMENT;
    Guard g(m->device);
    cudaStream_t st = (cudaStream_t)stream;
    const int rc = launch_grad(m, features, targets, n, st);
    if (rc != AKUA_OK) return rc;
    ++m->adam_steps;
    const float b1 = 0.9f, b2 = 0.999f;
    const float bc1 = (float)(1.0 - std::pow((double)b1, (double)m->adam_steps));
    const float bc2 = (float)(1.0 - std::pow((double)b2, (double)m->adam_steps));
    const int blocks = (akua::mlp::kParams + 1 + 255) / 256;
    akua::mlp::k_mlp_adam<<<blocks, 256, 0, st>>>(m->params, m->grad, m->m, m->v, learningRate,
                                                 b1, b2, 1e-8f, bc1, bc2);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) {  // the forward pass reads the updated weights from their image
        akua::mlp::k_mlp_image<<<1, akua::mlp::kThreads, 0, st>>>(m->params, m->image);
        e = cudaGetLastError();
    }
    return status_of(e);
}

int akua_mlp_synchronize(akua_mlp* m, void* stream) {
    if (!m) return AKUA_ERR_INVALID_ARGUMENT;
    Guard g(m->device);
    uint32_t err = 0;
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaMemcpy(&err, m->err, sizeof(err), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return status_of(e);
    return err ? AKUA_ERR_DEVICE_CHECK : AKUA_OK;
}

}  // extern "C"
