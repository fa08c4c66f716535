// TEST INFRASTRUCTURE ONLY.  Compiles the reference's own smoothing-kernel and cross-product
// helpers (include/AkuaEngine/CUDA/SmoothingKernelsCUDA.h:16-28, MathUtilsCUDA.h:12-18) unchanged
// on the host and prints known-answer values as float bit patterns, one JSON object per line.
// Built into oracle/_ref/ by oracle/ref_kat.py; the values are committed under tests/golden/.
#include <AkuaEngine/CUDA/MathUtilsCUDA.h>
#include <AkuaEngine/CUDA/SmoothingKernelsCUDA.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <initializer_list>

static uint32_t bits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

int main() {
    using namespace AkuaEngine;
    const float hs[] = {0.1f, 0.05f, 0.2f, 0.0375f};
    for (float h : hs) {
        const float h2 = h * h;
        for (int k = 0; k <= 40; ++k) {
            const float r2 = h2 * (float)k / 32.0f;  // includes r2 > h2 (zero branch)
            const float w = SmoothingKernels::device_poly6(r2, h);
            std::printf("{\"fn\":\"poly6\",\"h\":%u,\"r2\":%u,\"out\":[%u]}\n", bits(h), bits(r2), bits(w));
        }
        uint32_t state = 12345u;
        for (int k = 0; k < 64; ++k) {
            float v[3];
            for (float& c : v) {
                state = state * 1664525u + 1013904223u;
                c = ((float)(state >> 8) / 16777216.0f - 0.5f) * 2.4f * h;
            }
            if (k == 0) { v[0] = 0.f; v[1] = 0.f; v[2] = 0.f; }            // |r| < 1e-5
            if (k == 1) { v[0] = h; v[1] = 0.f; v[2] = 0.f; }              // |r| == h
            if (k == 2) { v[0] = 0.5f * h; v[1] = 0.f; v[2] = 0.f; }
            const glm::vec3 g = SmoothingKernels::device_gradient_spiky(glm::vec3(v[0], v[1], v[2]), h);
            std::printf("{\"fn\":\"spiky\",\"h\":%u,\"r\":[%u,%u,%u],\"out\":[%u,%u,%u]}\n", bits(h),
                        bits(v[0]), bits(v[1]), bits(v[2]), bits(g.x), bits(g.y), bits(g.z));
        }
    }
    uint32_t state = 777u;
    for (int k = 0; k < 32; ++k) {
        float a[3], b[3];
        for (float* arr : {a, b})
            for (int c = 0; c < 3; ++c) {
                state = state * 1664525u + 1013904223u;
                arr[c] = ((float)(state >> 8) / 16777216.0f - 0.5f) * 8.0f;
            }
        const glm::vec3 c = MathUtilsCUDA::cross(glm::vec3(a[0], a[1], a[2]), glm::vec3(b[0], b[1], b[2]));
        std::printf("{\"fn\":\"cross\",\"a\":[%u,%u,%u],\"b\":[%u,%u,%u],\"out\":[%u,%u,%u]}\n",
                    bits(a[0]), bits(a[1]), bits(a[2]), bits(b[0]), bits(b[1]), bits(b[2]),
                    bits(c.x), bits(c.y), bits(c.z));
    }
    return 0;
}
