// Device-side parameters and pair math of the PBF step.
//
// Compiled with --fmad=false: no multiply-add is fused unless written as __fmaf_rn.  The explicit
// fusions below are the ones the CUDA compiler applies by default to the reference's expressions
// (a product whose only use is an addend: a*b + c -> fma(a, b, c); for a sum of two products the
// first product is fused), so a step here rounds like the reference's wherever it uses the same
// operations.  The reference's powf calls with integer exponents (SmoothingKernelsCUDA.h:20,27 and
// the artificial-pressure power, ConstraintSolverCUDA.cu:124) are multiplications here.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace akua {

// Everything a kernel of one step reads besides the particle arrays.  Lives in device memory and is
// rewritten by a one-thread kernel at the start of every step, so a captured step graph replays
// with new dt / box / gravity without re-capture.
// Solid obstacles as signed distance functions (SDF boundary; the reference's clamp is a stand-in
// for a boundary of this kind, ConstraintSolverCUDA.cu:131-134).  type: 1 sphere (centre a,
// radius), 2 axis-aligned box (centre a, half extents b, corner radius), 3 capsule (segment a-b,
// radius), 4 half-space (unit normal a pointing into the fluid, offset b[0]: solid where
// a . x < b[0]).
struct SdfShape {
    int32_t type;
    float a[3];
    float b[3];
    float radius;
};
enum { kSdfSphere = 1, kSdfBox = 2, kSdfCapsule = 3, kSdfPlane = 4 };

struct StepParams {
    // PBFConfig-derived constants
    float h;            // smoothRadius
    float h2;           // h*h in float (SmoothingKernelsCUDA.h:17, NeighbourSearchCUDA.cu:90)
    float kp;           // 315 / (64 * 3.14f * h^9), evaluated in double and rounded
    float ks;           // -45 / (3.14f * h^6), evaluated in double and rounded
    float w0;           // poly6(0)
    float inv_rho0;     // 1.0f / restDensity (ConstraintSolverCUDA.cu:201)
    float relaxation;
    float wdq;          // poly6(delta_q^2)
    float inv_wdq;      // 1 / wdq (fast math only)
    float neg_k;        // -k
    float corr_n;       // n (float)
    int32_t corr_n_int; // n when it is an integer in [0, 64], else -1
    float hash_cell;    // cell size of the hash keys (smoothRadius, NeighbourSearchCUDA.cu:163)
    float search_cell;  // cell size of the neighbour walk (spatialHashCellSize)
    float vort_eps;
    float visc;
    // per step
    float dt;
    float gravity[3];
    float box_min[3];
    float box_max[3];
    float neg_restitution;  // -e
    float keep;             // 1 - friction, in float
    // sizes
    int32_t n;
    int32_t cap;
    uint32_t table_size;
    uint64_t table_magic;   // floor((2^64 - 1) / table_size) + 1, for the exact u32 modulo
    // Morton key of the walk cell: cell - sp_origin per axis, clamped to sp_bits bits
    int32_t sp_origin[3];
    int32_t sp_bits;
    // Batches of independent scenes: this scene's index, its first bucket in the shared table
    // (hash keys are table_offset + hash, so one sort orders by (scene, hash)), and the scene of
    // every particle (null for a single scene).  Scenes occupy the same index range in every
    // particle order (import, reference, internal), so one array serves all kernels.
    int32_t scene;
    uint32_t table_offset;
    const uint16_t* scene_of;
    // SDF obstacles (none: the reference's box clamp alone)
    const SdfShape* shapes;
    int32_t num_shapes;
    float sdf_min_dist;
    float sdf_stiffness;
};

// The parameters of the scene particle (or reference rank, or internal slot) i belongs to.
__device__ __forceinline__ const StepParams& params_for(const StepParams* P, int i) {
    const uint16_t* sid = P->scene_of;
    return sid ? P[sid[i]] : *P;
}

__device__ __forceinline__ float fmaf_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }

// glm::dot(vec3, vec3) = tmp.x + tmp.y + tmp.z with tmp = a*b, contracted.
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
    return __fmaf_rn(az, bz, __fmaf_rn(ax, bx, ay * by));
}
__device__ __forceinline__ float len2(float x, float y, float z) { return dot3(x, y, z, x, y, z); }

// MathUtilsCUDA::cross, contracted: fma(a.y, b.z, -(a.z*b.y)) etc.
__device__ __forceinline__ float3 cross3(float ax, float ay, float az, float bx, float by, float bz) {
    return make_float3(__fmaf_rn(ay, bz, -(az * by)), __fmaf_rn(az, bx, -(ax * bz)),
                       __fmaf_rn(ax, by, -(ay * bx)));
}

// Cell coordinate: floorf(x / cell) with an IEEE divide (NeighbourSearchCUDA.cu:15-21).
__device__ __forceinline__ int cell_coord(float x, float cell) {
    return static_cast<int>(floorf(__fdiv_rn(x, cell)));
}

// a % d for any u32 a and d >= 1, with magic = floor((2^64 - 1) / d) + 1 (Lemire, Kaser and Kurz,
// "Faster remainder by direct computation", 2019): the low 64 bits of magic * a hold the
// fractional part of a / d, and its product with d carries the remainder in the high word.
__device__ __forceinline__ uint32_t fast_mod(uint32_t a, uint64_t magic, uint32_t d) {
    const uint64_t low = magic * (uint64_t)a;
    return (uint32_t)__umul64hi(low, (uint64_t)d);
}

// NeighbourSearchCUDA.cu:23-27: int products wrap, u32 xor, then % tableSize as u32.
__device__ __forceinline__ uint32_t cell_hash(int cx, int cy, int cz, uint32_t table,
                                              uint64_t magic) {
    const uint32_t hx = static_cast<uint32_t>(cx) * 73856093u;
    const uint32_t hy = static_cast<uint32_t>(cy) * 19349663u;
    const uint32_t hz = static_cast<uint32_t>(cz) * 83492791u;
    return fast_mod(hx ^ hy ^ hz, magic, table);
}

// Signed distance from the solid of shape s (positive on the fluid side) and its unit gradient,
// in plain IEEE single operations (no contraction); the host restatement uses the same ones.
__device__ __forceinline__ float sdf_eval(const SdfShape& s, float x, float y, float z, float* n) {
    if (s.type == kSdfPlane) {
        n[0] = s.a[0]; n[1] = s.a[1]; n[2] = s.a[2];
        return (s.a[0] * x + s.a[1] * y + s.a[2] * z) - s.b[0];
    }
    float dx, dy, dz;
    if (s.type == kSdfBox) {
        const float px = x - s.a[0], py = y - s.a[1], pz = z - s.a[2];
        const float qx = fabsf(px) - s.b[0], qy = fabsf(py) - s.b[1], qz = fabsf(pz) - s.b[2];
        const float ox = fmaxf(qx, 0.f), oy = fmaxf(qy, 0.f), oz = fmaxf(qz, 0.f);
        const float lo = __fsqrt_rn(ox * ox + oy * oy + oz * oz);
        const float qm = fmaxf(qx, fmaxf(qy, qz));
        if (lo > 0.f) {
            n[0] = __fdiv_rn(copysignf(ox, px), lo);
            n[1] = __fdiv_rn(copysignf(oy, py), lo);
            n[2] = __fdiv_rn(copysignf(oz, pz), lo);
        } else {  // inside: out through the nearest face (x before y before z on ties)
            n[0] = n[1] = n[2] = 0.f;
            const int k = (qx == qm) ? 0 : ((qy == qm) ? 1 : 2);
            const float pk = k == 0 ? px : (k == 1 ? py : pz);
            n[k] = pk < 0.f ? -1.f : 1.f;
        }
        return (lo + fminf(qm, 0.f)) - s.radius;
    }
    if (s.type == kSdfCapsule) {
        const float ux = s.b[0] - s.a[0], uy = s.b[1] - s.a[1], uz = s.b[2] - s.a[2];
        const float wx = x - s.a[0], wy = y - s.a[1], wz = z - s.a[2];
        const float uu = ux * ux + uy * uy + uz * uz;
        float t = uu > 0.f ? __fdiv_rn(wx * ux + wy * uy + wz * uz, uu) : 0.f;
        t = fminf(fmaxf(t, 0.f), 1.f);
        dx = wx - t * ux; dy = wy - t * uy; dz = wz - t * uz;
    } else {  // sphere
        dx = x - s.a[0]; dy = y - s.a[1]; dz = z - s.a[2];
    }
    const float l = __fsqrt_rn(dx * dx + dy * dy + dz * dz);
    if (l > 0.f) {
        n[0] = __fdiv_rn(dx, l); n[1] = __fdiv_rn(dy, l); n[2] = __fdiv_rn(dz, l);
    } else {
        n[0] = 0.f; n[1] = 1.f; n[2] = 0.f;
    }
    return l - s.radius;
}

// Pushes a corrected position out of every obstacle it comes within sdf_min_dist of (soft, like
// the box clamp): x += stiffness * (min_dist - phi) * grad phi, shapes in order.
__device__ __forceinline__ void sdf_correct(const StepParams& p, float& x, float& y, float& z) {
    for (int k = 0; k < p.num_shapes; ++k) {
        float n[3];
        const float phi = sdf_eval(p.shapes[k], x, y, z, n);
        if (phi < p.sdf_min_dist) {
            const float c = p.sdf_stiffness * (p.sdf_min_dist - phi);
            x = x + c * n[0];
            y = y + c * n[1];
            z = z + c * n[2];
        }
    }
}

// poly6 (SmoothingKernelsCUDA.h:16-21): 0 when r2 > h2, else kp * (h2 - r2)^3.
__device__ __forceinline__ float poly6(const StepParams& p, float r2) {
    const float d = p.h2 - r2;
    const float w = p.kp * ((d * d) * d);
    return r2 > p.h2 ? 0.0f : w;
}

// Integer power by binary exponentiation (same multiplication pattern as the host restatement).
__device__ __forceinline__ float pown(float x, int n) {
    float result = 1.0f;
    float base = x;
    bool first = true;
    while (n > 0) {
        if (n & 1) {
            result = first ? base : result * base;
            first = false;
        }
        n >>= 1;
        if (n) base = base * base;
    }
    return result;
}

}  // namespace akua
