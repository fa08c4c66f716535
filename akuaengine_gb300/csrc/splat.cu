// Headless point-splat renderer of the particle records: the consumer of the reference's interop
// buffer, restated as CUDA kernels writing an RGBA8 image (no graphics API).
//
// What it computes is the reference's particle pass (assets/shaders/fluidParticle.vert/.frag,
// src/Rendering/Renderer.cpp:29-50, src/Application/Application.cpp:72,112-113):
//   vertex   world = position (the particle object's model matrix is the identity,
//            SceneObject.cpp:61-62); point size = size / |world - camera|;
//            clip = (projection * view) * world
//   raster   a non-antialiased point: the pixels whose centres lie in the square of that side
//            around the window position; points whose vertex is outside the clip volume vanish
//   fragment offset = pointCoord - 0.5 (pointCoord's origin at the upper left); discarded when
//            |offset| > 0.5; colour = particle colour * exp(-|offset|^2 * 3)
//   output   depth test LESS against a cleared depth of 1, no blending, clear colour
//            (0.15, 0.15, 0.18, 1); equal depths keep the first particle drawn (lowest index)
// view = lookAt(eye, eye + gaze, up) and projection = perspective(fovy, aspect, near, far) are the
// right-handed, [-1, 1]-depth conventions of the reference's camera (Camera.cpp:32,74-87,
// Renderer.cpp:30).
//
// Pass 1 projects each particle; pass 2 (one warp per particle) resolves visibility per pixel with
// one 64-bit atomicMin of (depth bits, particle index) -- non-negative float depths order like
// their bit patterns, and the index breaks ties as draw order does; pass 3 shades each pixel from
// its winning particle.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <new>

#include "akua_pbf.h"

namespace {

struct SplatParams {
    float vp[16];   // projection * view, column-major (vp[4 * col + row])
    float eye[3];
    int width, height;
};

constexpr unsigned long long kEmpty = ~0ull;
constexpr float kMaxPointSize = 2047.0f;  // a typical implementation's point size range

__device__ __forceinline__ float frag_alpha(float ox, float oy, float* dist_out) {
    const float dist = sqrtf(ox * ox + oy * oy);
    *dist_out = dist;
    return expf(-dist * dist * 3.0f);
}

// proj[i] = (window x, window y, window depth, point size); size 0 marks a clipped point.
__global__ void k_splat_project(SplatParams P, const char* __restrict__ aos, uint64_t stride,
                                int n, float4* __restrict__ proj, float4* __restrict__ col) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* r = reinterpret_cast<const float*>(aos + (uint64_t)i * stride);
    const float x = r[0], y = r[1], z = r[2];
    const float dx = x - P.eye[0], dy = y - P.eye[1], dz = z - P.eye[2];
    const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
    float size = r[26] / dist;  // Particle::size follows colour (offset 104 bytes)
    size = fminf(fmaxf(size, 1.0f), kMaxPointSize);
    float c[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) c[k] = P.vp[k] * x + P.vp[4 + k] * y + P.vp[8 + k] * z + P.vp[12 + k];
    const float w = c[3];
    const bool inside = w > 0.0f && fabsf(c[0]) <= w && fabsf(c[1]) <= w && fabsf(c[2]) <= w;
    const float nx = c[0] / w, ny = c[1] / w, nz = c[2] / w;
    const float xw = (nx + 1.0f) * 0.5f * (float)P.width;
    const float yw = (ny + 1.0f) * 0.5f * (float)P.height;
    const float zw = (nz + 1.0f) * 0.5f;
    proj[i] = make_float4(xw, yw, zw, inside ? size : 0.0f);
    col[i] = make_float4(r[22], r[23], r[24], r[25]);
}

// Pixel span of a point: centres px + 0.5 in [xw - s/2, xw + s/2).
__device__ __forceinline__ void span(float c, float s, int limit, int* lo, int* hi) {
    *lo = max(0, (int)ceilf(c - 0.5f * s - 0.5f));
    *hi = min(limit - 1, (int)ceilf(c + 0.5f * s - 0.5f) - 1);
}

__global__ void k_splat_raster(SplatParams P, const float4* __restrict__ proj, int n,
                               unsigned long long* __restrict__ zbuf) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    const float4 q = proj[warp];
    if (q.w <= 0.0f || !(q.z < 1.0f)) return;  // clipped, or not nearer than the cleared depth
    int x0, x1, y0, y1;
    span(q.x, q.w, P.width, &x0, &x1);
    span(q.y, q.w, P.height, &y0, &y1);
    if (x0 > x1 || y0 > y1) return;
    const int nxp = x1 - x0 + 1;
    const int count = nxp * (y1 - y0 + 1);
    const unsigned long long key =
        ((unsigned long long)__float_as_uint(fmaxf(q.z, 0.0f)) << 32) | (unsigned)warp;
    for (int k = lane; k < count; k += 32) {
        const int px = x0 + k % nxp, py = y0 + k / nxp;
        const float ox = (((float)px + 0.5f) - q.x) / q.w;   // pointCoord.s - 0.5
        const float oy = -(((float)py + 0.5f) - q.y) / q.w;  // pointCoord.t - 0.5 (t downwards)
        float dist;
        frag_alpha(ox, oy, &dist);
        if (dist > 0.5f) continue;
        atomicMin(&zbuf[(size_t)py * P.width + px], key);
    }
}

__device__ __forceinline__ uint32_t to_u8(float v) {
    return (uint32_t)(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f + 0.5f);
}

// Row 0 of the image is the top of the window (window y = height - 1).
__global__ void k_splat_resolve(SplatParams P, const float4* __restrict__ proj,
                                const float4* __restrict__ col,
                                const unsigned long long* __restrict__ zbuf,
                                uint32_t* __restrict__ rgba) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P.width * P.height) return;
    const int px = p % P.width, py = p / P.width;
    const unsigned long long key = zbuf[p];
    float c[4] = {0.15f, 0.15f, 0.18f, 1.0f};
    if (key != kEmpty) {
        const int i = (int)(key & 0xFFFFFFFFull);
        const float4 q = proj[i];
        const float4 k = col[i];
        const float ox = (((float)px + 0.5f) - q.x) / q.w;
        const float oy = -(((float)py + 0.5f) - q.y) / q.w;
        float dist;
        const float a = frag_alpha(ox, oy, &dist);
        c[0] = k.x * a;
        c[1] = k.y * a;
        c[2] = k.z * a;
        c[3] = k.w * a;
    }
    rgba[(size_t)(P.height - 1 - py) * P.width + px] =
        to_u8(c[0]) | (to_u8(c[1]) << 8) | (to_u8(c[2]) << 16) | (to_u8(c[3]) << 24);
}

int status_of(cudaError_t e) {
    if (e == cudaSuccess) return AKUA_OK;
    if (e == cudaErrorMemoryAllocation) return AKUA_ERR_OUT_OF_MEMORY;
    return AKUA_ERR_CUDA;
}

// column-major 4x4 helpers in double
void mat_mul(const double* a, const double* b, double* out) {  // out = a * b
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            double s = 0.0;
            for (int k = 0; k < 4; ++k) s += a[4 * k + r] * b[4 * c + k];
            out[4 * c + r] = s;
        }
}

void normalize3(double* v) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int k = 0; k < 3; ++k) v[k] /= l;
}

void cross3(const double* a, const double* b, double* out) {
    out[0] = a[1] * b[2] - a[2] * b[1];
    out[1] = a[2] * b[0] - a[0] * b[2];
    out[2] = a[0] * b[1] - a[1] * b[0];
}

bool finite_camera(const akua_camera* c) {
    for (int k = 0; k < 3; ++k)
        if (!std::isfinite(c->position[k]) || !std::isfinite(c->gaze[k]) || !std::isfinite(c->up[k]))
            return false;
    return std::isfinite(c->fovDegrees) && c->fovDegrees > 0.0f && c->fovDegrees < 180.0f &&
           c->nearZ > 0.0f && c->farZ > c->nearZ;
}

}  // namespace

struct akua_splat {
    int device = 0;
    int width = 0, height = 0;
    unsigned long long* zbuf = nullptr;
    float4* proj = nullptr;
    float4* col = nullptr;
    int capacity = 0;  // particles proj/col can hold
};

extern "C" {

void akua_camera_default(akua_camera* c) {
    if (!c) return;
    // CameraConfig.h:8-16 (yaw -90, pitch 0: gaze (0, 0, -1)); Application.cpp:17-18
    c->position[0] = 3.0f; c->position[1] = 2.0f; c->position[2] = 6.0f;
    c->gaze[0] = 0.0f; c->gaze[1] = 0.0f; c->gaze[2] = -1.0f;
    c->up[0] = 0.0f; c->up[1] = 1.0f; c->up[2] = 0.0f;
    c->fovDegrees = 45.0f;
    c->nearZ = 0.1f;
    c->farZ = 160.0f;
}

int akua_camera_matrices(const akua_camera* cam, float aspect, float* view, float* projection,
                         float* viewProjection) {
    if (!cam || !finite_camera(cam) || !(aspect > 0.0f)) return AKUA_ERR_INVALID_ARGUMENT;
    double f[3] = {cam->gaze[0], cam->gaze[1], cam->gaze[2]};
    normalize3(f);
    double wu[3] = {cam->up[0], cam->up[1], cam->up[2]};
    double s[3], u[3];
    cross3(f, wu, s);
    normalize3(s);
    cross3(s, f, u);
    const double e[3] = {cam->position[0], cam->position[1], cam->position[2]};
    double V[16] = {0};
    for (int k = 0; k < 3; ++k) {
        V[4 * k + 0] = s[k];
        V[4 * k + 1] = u[k];
        V[4 * k + 2] = -f[k];
    }
    V[12] = -(s[0] * e[0] + s[1] * e[1] + s[2] * e[2]);
    V[13] = -(u[0] * e[0] + u[1] * e[1] + u[2] * e[2]);
    V[14] = f[0] * e[0] + f[1] * e[1] + f[2] * e[2];
    V[15] = 1.0;
    const double t = std::tan(0.5 * (double)cam->fovDegrees * 3.14159265358979323846 / 180.0);
    const double zn = cam->nearZ, zf = cam->farZ;
    double Pm[16] = {0};
    Pm[0] = 1.0 / ((double)aspect * t);
    Pm[5] = 1.0 / t;
    Pm[10] = -(zf + zn) / (zf - zn);
    Pm[11] = -1.0;
    Pm[14] = -(2.0 * zf * zn) / (zf - zn);
    double VP[16];
    mat_mul(Pm, V, VP);
    for (int k = 0; k < 16; ++k) {
        if (view) view[k] = (float)V[k];
        if (projection) projection[k] = (float)Pm[k];
        if (viewProjection) viewProjection[k] = (float)VP[k];
    }
    return AKUA_OK;
}

int akua_splat_create(int32_t width, int32_t height, akua_splat** out) {
    if (!out || width <= 0 || height <= 0 || (int64_t)width * height > (1ll << 28))
        return AKUA_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    akua_splat* r = new (std::nothrow) akua_splat();
    if (!r) return AKUA_ERR_OUT_OF_MEMORY;
    r->width = width;
    r->height = height;
    cudaGetDevice(&r->device);
    const cudaError_t e = cudaMalloc(&r->zbuf, sizeof(unsigned long long) * (size_t)width * height);
    if (e != cudaSuccess) {
        delete r;
        cudaGetLastError();
        return status_of(e);
    }
    *out = r;
    return AKUA_OK;
}

int akua_splat_destroy(akua_splat* r) {
    if (!r) return AKUA_ERR_INVALID_ARGUMENT;
    cudaDeviceSynchronize();
    cudaFree(r->zbuf);
    cudaFree(r->proj);
    cudaFree(r->col);
    delete r;
    return AKUA_OK;
}

int akua_splat_render(akua_splat* r, const void* particles, size_t stride, int32_t n,
                      const akua_camera* camera, uint32_t* rgba, void* stream) {
    if (!r || !camera || !rgba || n < 0 || (n > 0 && !particles) ||
        stride < sizeof(akua_particle) || stride % 4 != 0)
        return AKUA_ERR_INVALID_ARGUMENT;
    SplatParams P{};
    P.width = r->width;
    P.height = r->height;
    int rc = akua_camera_matrices(camera, (float)r->width / (float)r->height, nullptr, nullptr,
                                  P.vp);
    if (rc != AKUA_OK) return rc;
    for (int k = 0; k < 3; ++k) P.eye[k] = camera->position[k];
    cudaStream_t st = (cudaStream_t)stream;
    if (n > r->capacity) {
        cudaError_t e = cudaStreamSynchronize(st);
        cudaFree(r->proj);
        cudaFree(r->col);
        r->proj = nullptr;
        r->col = nullptr;
        r->capacity = 0;
        if (e == cudaSuccess) e = cudaMalloc(&r->proj, sizeof(float4) * (size_t)n);
        if (e == cudaSuccess) e = cudaMalloc(&r->col, sizeof(float4) * (size_t)n);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return status_of(e);
        }
        r->capacity = n;
    }
    const size_t pixels = (size_t)r->width * r->height;
    cudaError_t e = cudaMemsetAsync(r->zbuf, 0xFF, sizeof(unsigned long long) * pixels, st);
    if (e != cudaSuccess) return status_of(e);
    if (n > 0) {
        k_splat_project<<<(n + 255) / 256, 256, 0, st>>>(P, static_cast<const char*>(particles),
                                                          stride, n, r->proj, r->col);
        const long long threads = 32ll * n;
        k_splat_raster<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(P, r->proj, n, r->zbuf);
    }
    k_splat_resolve<<<(unsigned)((pixels + 255) / 256), 256, 0, st>>>(P, r->proj, r->col, r->zbuf,
                                                                       rgba);
    return status_of(cudaGetLastError());
}

}  // extern "C"
