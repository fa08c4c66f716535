// TEST INFRASTRUCTURE ONLY — never linked into, loaded by, or called from the product path.
//
// CPU oracle for the Position-Based Fluids step of AkuaEngine (`PBFSolver::step`,
// src/Simulation/PBFSolver.cpp:22-78).  It restates the reference's algorithm on the host:
//   predict            src/CUDA/IntegrationCUDA.cu:27-36
//   cell + hash        src/CUDA/NeighbourSearchCUDA.cu:15-27, 36-44 (cell size = smoothRadius, :163)
//   sort by hash       src/CUDA/NeighbourSearchCUDA.cu:167-170 (stable: ties keep the previous order)
//   bucket starts      src/CUDA/NeighbourSearchCUDA.cu:52-65
//   neighbour walk     src/CUDA/NeighbourSearchCUDA.cu:72-130 (cell size = spatialHashCellSize)
//   density            src/CUDA/ConstraintSolverCUDA.cu:16-42
//   lambda             src/CUDA/ConstraintSolverCUDA.cu:51-97
//   position delta     src/CUDA/ConstraintSolverCUDA.cu:99-130
//   correct + clamp    src/CUDA/ConstraintSolverCUDA.cu:136-169
//   update             src/CUDA/IntegrationCUDA.cu:38-49
//   boundary damping   src/CUDA/IntegrationCUDA.cu:51-102 (called with e=0, f=0.95, PBFSolver.cpp:64)
//   vorticity          src/CUDA/IntegrationCUDA.cu:104-128
//   confinement        src/CUDA/IntegrationCUDA.cu:130-165
//   XSPH               src/CUDA/IntegrationCUDA.cu:167-195 (read from a velocity snapshot; the
//                      reference reads neighbours' velocities while other threads overwrite them)
//   poly6 / spiky      include/AkuaEngine/CUDA/SmoothingKernelsCUDA.h:16-28 (pi written as 3.14f)
//   SDF obstacles      not in the reference (it plans a boundary in place of its clamp,
//                      ConstraintSolverCUDA.cu:131-134): applied after the box clamp and after
//                      the six-plane damping, in plain single operations
//   cross              include/AkuaEngine/CUDA/MathUtilsCUDA.h:12-18
//
// Arithmetic.  Every product-sum that the CUDA compiler contracts by default in the reference
// source (a*b+c with a single-use product) is written here as an explicit fused multiply-add
// when ORACLE_FMA is set, and as two rounded operations otherwise.  The file must be compiled
// with -ffp-contract=off so the compiler adds no contraction of its own.  `powf(x, 2|3)` and the
// integer-exponent `powf` of the artificial pressure are evaluated by multiplication, and the
// kernel constants 315/(64*3.14*h^9) and 45/(3.14*h^6) are evaluated once in double precision and
// rounded, so results differ from a powf-based evaluation by a few units in the last place.
//
// ORACLE_FP64 runs the same equations after the neighbour search in double precision (the grid,
// hashes and lists still come from the float predicted positions) to measure FP32 error.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct ParticleRec {  // include/AkuaEngine/Simulation/Particle.h:8-31 (108 bytes, 4-byte aligned)
    float position[3];
    float velocity[3];
    float new_position[3];
    float new_velocity[3];
    float position_delta[3];
    float vorticity[3];
    float mass;
    float density;
    float lambda;
    uint32_t hash;
    float color[4];
    float size;
};
static_assert(sizeof(ParticleRec) == 108, "Particle record must be 108 bytes");

}  // namespace

extern "C" {

struct OracleParams {
    float rest_density;       // PBFConfig::restDensity
    float smooth_radius;      // PBFConfig::smoothRadius (also the hashing cell, NeighbourSearchCUDA.cu:163)
    float cell_size;          // PBFConfig::spatialHashCellSize (neighbour walk cell)
    float relaxation;         // PBFConfig::relaxation
    float vorticity_epsilon;  // PBFConfig::vorticityEpsilon
    float viscosity;          // PBFConfig::viscosity (XSPH c)
    int32_t max_neighbours;   // PBFConfig::maxNeighbours
    int32_t solver_iterations;
    float gravity[3];
    float corr_k, corr_n, corr_delta_q;  // LambdaCorrParams
    int32_t table_size;       // PBFSolver::_tableSize = maxNeighbours * numParticles
    float dt;
    float box_min[3];
    float box_max[3];
    float restitution;        // 0 at the reference call site
    float friction;           // 0.95 at the reference call site
    uint32_t flags;
    int32_t num_threads;      // <= 0: OpenMP default
    int32_t num_shapes;       // SDF obstacles (0: none)
    float sdf_min_dist;
    float sdf_stiffness;
    int32_t pad_;
    const struct OracleShape* shapes;
};

struct OracleShape {  // type 1 sphere, 2 box, 3 capsule, 4 half-space (see sdf_eval)
    int32_t type;
    float a[3];
    float b[3];
    float radius;
};

enum { ORACLE_FMA = 1u, ORACLE_FP64 = 2u };

}  // extern "C"

namespace {

template <bool FMA, class R>
inline R fmac(R a, R b, R c) {
    if constexpr (FMA) return std::fma(a, b, c);
    else return a * b + c;
}

template <class R>
struct V3 {
    R x, y, z;
};

template <class R>
inline V3<R> sub(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }

// glm::dot for vec3: tmp = a*b; tmp.x + tmp.y + tmp.z (glm/detail/func_geometric.inl).  Under
// contraction the first product is fused into the first sum and the third into the second.
template <bool FMA, class R>
inline R dot3(V3<R> a, V3<R> b) {
    if constexpr (FMA) return std::fma(a.z, b.z, std::fma(a.x, b.x, a.y * b.y));
    else return (a.x * b.x + a.y * b.y) + a.z * b.z;
}

// MathUtilsCUDA::cross: a.y*b.z - a.z*b.y, ... — contracted as fma(a.y, b.z, -(a.z*b.y)).
template <bool FMA, class R>
inline V3<R> cross3(V3<R> a, V3<R> b) {
    if constexpr (FMA)
        return {std::fma(a.y, b.z, -(a.z * b.y)), std::fma(a.z, b.x, -(a.x * b.z)),
                std::fma(a.x, b.y, -(a.y * b.x))};
    else
        return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}

// Integer power by binary exponentiation; the same multiplication pattern is used on the device.
template <class R>
inline R pown(R x, int n) {
    R result = R(1);
    R base = x;
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

struct Consts {
    double poly6;   // 315 / (64 * 3.14f * h^9)
    double spiky;   // -45 / (3.14f * h^6)
};

Consts kernel_consts(float h_f) {
    const double pi_ref = (double)3.14f;  // the reference writes pi as the float literal 3.14f
    const double h = (double)h_f;
    const double h2 = h * h, h3 = h2 * h, h6 = h3 * h3, h9 = h6 * h3;
    Consts c;
    c.poly6 = 315.0 / (64.0 * pi_ref * h9);
    c.spiky = -(45.0 / (pi_ref * h6));
    return c;
}

inline uint32_t cell_hash(int cx, int cy, int cz, uint32_t table) {
    // NeighbourSearchCUDA.cu:23-27: int products wrap, then u32 xor, then % tableSize (as u32).
    const uint32_t hx = (uint32_t)cx * 73856093u;
    const uint32_t hy = (uint32_t)cy * 19349663u;
    const uint32_t hz = (uint32_t)cz * 83492791u;
    return (hx ^ hy ^ hz) % table;
}

inline int cell_coord(float x, float cell) { return (int)std::floor(x / cell); }

template <bool FMA, class R>
struct Kernels {
    R h, h2, kp, ks, eps_r;
    R poly6(R r2) const {
        if (r2 > h2) return R(0);
        const R d = h2 - r2;
        return kp * ((d * d) * d);
    }
    V3<R> spiky(V3<R> rv) const {
        const R r = std::sqrt(dot3<FMA>(rv, rv));
        if (r > h || r < eps_r) return {R(0), R(0), R(0)};
        const R q = h - r;
        const R c = ks * (q * q);
        return {(c * rv.x) / r, (c * rv.y) / r, (c * rv.z) / r};
    }
};

template <bool FMA, class R>
Kernels<FMA, R> make_kernels(float h_f) {
    Consts c = kernel_consts(h_f);
    Kernels<FMA, R> k;
    k.h = (R)h_f;
    k.h2 = (R)h_f * (R)h_f;
    k.kp = (R)c.poly6;
    k.ks = (R)c.spiky;
    k.eps_r = (R)1e-5f;
    return k;
}

struct Grid {
    std::vector<uint32_t> nbr;  // n * cap, row-major (reference layout i*cap + k)
    std::vector<uint32_t> cnt;
};

// Signed distance from an obstacle (positive in the fluid) and its unit gradient.
template <class R>
R sdf_eval(const OracleShape& s, R x, R y, R z, R* n) {
    const R a0 = s.a[0], a1 = s.a[1], a2 = s.a[2];
    if (s.type == 4) {
        n[0] = a0; n[1] = a1; n[2] = a2;
        return (a0 * x + a1 * y + a2 * z) - (R)s.b[0];
    }
    R dx, dy, dz;
    if (s.type == 2) {
        const R px = x - a0, py = y - a1, pz = z - a2;
        const R qx = std::fabs(px) - (R)s.b[0], qy = std::fabs(py) - (R)s.b[1],
                qz = std::fabs(pz) - (R)s.b[2];
        const R ox = std::fmax(qx, R(0)), oy = std::fmax(qy, R(0)), oz = std::fmax(qz, R(0));
        const R lo = std::sqrt(ox * ox + oy * oy + oz * oz);
        const R qm = std::fmax(qx, std::fmax(qy, qz));
        if (lo > R(0)) {
            n[0] = std::copysign(ox, px) / lo;
            n[1] = std::copysign(oy, py) / lo;
            n[2] = std::copysign(oz, pz) / lo;
        } else {
            n[0] = n[1] = n[2] = R(0);
            const int k = (qx == qm) ? 0 : ((qy == qm) ? 1 : 2);
            const R pk = k == 0 ? px : (k == 1 ? py : pz);
            n[k] = pk < R(0) ? R(-1) : R(1);
        }
        return (lo + std::fmin(qm, R(0))) - (R)s.radius;
    }
    if (s.type == 3) {
        const R ux = (R)s.b[0] - a0, uy = (R)s.b[1] - a1, uz = (R)s.b[2] - a2;
        const R wx = x - a0, wy = y - a1, wz = z - a2;
        const R uu = ux * ux + uy * uy + uz * uz;
        R t = uu > R(0) ? (wx * ux + wy * uy + wz * uz) / uu : R(0);
        t = std::fmin(std::fmax(t, R(0)), R(1));
        dx = wx - t * ux; dy = wy - t * uy; dz = wz - t * uz;
    } else {
        dx = x - a0; dy = y - a1; dz = z - a2;
    }
    const R l = std::sqrt(dx * dx + dy * dy + dz * dz);
    if (l > R(0)) {
        n[0] = dx / l; n[1] = dy / l; n[2] = dz / l;
    } else {
        n[0] = R(0); n[1] = R(1); n[2] = R(0);
    }
    return l - (R)s.radius;
}

template <bool FMA>
void neighbour_search(const OracleParams& P, int n, const std::vector<ParticleRec>& ps, Grid& g) {
    const int cap = P.max_neighbours;
    const uint32_t table = (uint32_t)P.table_size;
    std::vector<uint32_t> keys(n);
    for (int i = 0; i < n; ++i) keys[i] = ps[i].hash;
    g.nbr.assign((size_t)n * cap, 0u);
    g.cnt.assign(n, 0u);
    const float h2 = P.smooth_radius * P.smooth_radius;
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
        const ParticleRec& pi = ps[i];
        const int cx = cell_coord(pi.new_position[0], P.cell_size);
        const int cy = cell_coord(pi.new_position[1], P.cell_size);
        const int cz = cell_coord(pi.new_position[2], P.cell_size);
        int count = 0;
        const size_t start = (size_t)i * cap;
        for (int dx = -1; dx <= 1; ++dx)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dz = -1; dz <= 1; ++dz) {
                    const uint32_t hh = cell_hash(cx + dx, cy + dy, cz + dz, table);
                    // bucket start: first sorted index carrying this hash (kernel_build_hash_table)
                    auto it = std::lower_bound(keys.begin(), keys.end(), hh);
                    if (it == keys.end() || *it != hh) continue;
                    int k = (int)(it - keys.begin());
                    while (k < n && count < cap) {
                        if (k == i) { ++k; continue; }
                        if (keys[k] != hh) break;
                        const ParticleRec& pk = ps[k];
                        V3<float> sep{pi.new_position[0] - pk.new_position[0],
                                      pi.new_position[1] - pk.new_position[1],
                                      pi.new_position[2] - pk.new_position[2]};
                        const float d2 = dot3<FMA>(sep, sep);
                        if (d2 < h2) g.nbr[start + count++] = (uint32_t)k;
                        ++k;
                    }
                }
        g.cnt[i] = (uint32_t)count;
    }
}

template <bool FMA, class R>
int step_impl(const OracleParams& P, int n, ParticleRec* particles, uint32_t* out_perm,
              uint32_t* out_nbr, uint32_t* out_cnt) {
    const float dt = P.dt;
    // 1. predict (kernel_predict_position): v* = v + g*dt; x* = x + v*dt, both contracted.
    std::vector<ParticleRec> pre(particles, particles + n);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        ParticleRec& p = pre[i];
        for (int a = 0; a < 3; ++a) {
            p.new_velocity[a] = fmac<FMA>(P.gravity[a], dt, p.velocity[a]);
            p.new_position[a] = fmac<FMA>(p.new_velocity[a], dt, p.position[a]);
        }
        // 2. hash (kernel_compute_hashes, called with the smoothing radius as the cell size)
        p.hash = cell_hash(cell_coord(p.new_position[0], P.smooth_radius),
                           cell_coord(p.new_position[1], P.smooth_radius),
                           cell_coord(p.new_position[2], P.smooth_radius), (uint32_t)P.table_size);
    }
    // 3. stable sort of whole records by hash (thrust::sort with a.hash < b.hash)
    std::vector<uint32_t> perm(n);
    std::iota(perm.begin(), perm.end(), 0u);
    std::stable_sort(perm.begin(), perm.end(),
                     [&](uint32_t a, uint32_t b) { return pre[a].hash < pre[b].hash; });
    std::vector<ParticleRec> ps(n);
    for (int s = 0; s < n; ++s) ps[s] = pre[perm[s]];
    if (out_perm) std::memcpy(out_perm, perm.data(), sizeof(uint32_t) * n);

    // 4. neighbour lists from the float predicted positions
    Grid grid;
    neighbour_search<FMA>(P, n, ps, grid);
    const int cap = P.max_neighbours;
    if (out_cnt) std::memcpy(out_cnt, grid.cnt.data(), sizeof(uint32_t) * n);
    if (out_nbr) std::memcpy(out_nbr, grid.nbr.data(), sizeof(uint32_t) * (size_t)n * cap);

    const Kernels<FMA, R> K = make_kernels<FMA, R>(P.smooth_radius);
    const bool fp64 = std::is_same<R, double>::value;

    // State in R precision.
    std::vector<V3<R>> x(n), xs(n), v(n), dp(n, V3<R>{0, 0, 0}), omega(n), vstar(n);
    std::vector<R> m(n), rho(n), lam(n);
    for (int i = 0; i < n; ++i) {
        const ParticleRec& p = ps[i];
        x[i] = {(R)p.position[0], (R)p.position[1], (R)p.position[2]};
        v[i] = {(R)p.velocity[0], (R)p.velocity[1], (R)p.velocity[2]};
        m[i] = (R)p.mass;
        rho[i] = (R)p.density;
        lam[i] = (R)p.lambda;
        dp[i] = {(R)p.position_delta[0], (R)p.position_delta[1], (R)p.position_delta[2]};
        if (fp64) {
            // same prediction evaluated in double
            for (int a = 0; a < 3; ++a) {
                const double nv = (double)p.velocity[a] + (double)P.gravity[a] * (double)dt;
                const double np = (double)p.position[a] + nv * (double)dt;
                (&xs[i].x)[a] = (R)np;
            }
        } else {
            xs[i] = {(R)p.new_position[0], (R)p.new_position[1], (R)p.new_position[2]};
        }
    }
    const R inv_rho0 = fp64 ? (R)(1.0 / (double)P.rest_density) : (R)(1.0f / P.rest_density);
    const R relax = (R)P.relaxation;
    const R w0 = K.poly6(R(0));
    const R dq2 = (R)P.corr_delta_q * (R)P.corr_delta_q;
    const R wdq = K.poly6(dq2);
    const R neg_k = -(R)P.corr_k;
    const bool n_int = std::floor(P.corr_n) == P.corr_n && P.corr_n >= 0.f && P.corr_n <= 64.f;
    const int n_i = (int)P.corr_n;
    const R md = (R)0.025f, stiff = (R)0.5f;
    std::vector<V3<R>> xs_next(n);

    auto nb = [&](int i, int k) { return (int)grid.nbr[(size_t)i * cap + k]; };

    // 5. Jacobi iterations (runConstraintSolverCUDA, ConstraintSolverCUDA.cu:206-218)
    for (int it = 0; it < P.solver_iterations; ++it) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {  // densities
            R r = m[i] * w0;
            for (uint32_t k = 0; k < grid.cnt[i]; ++k) {
                const int j = nb(i, k);
                const V3<R> sep = sub(xs[i], xs[j]);
                r = fmac<FMA>(m[j], K.poly6(dot3<FMA>(sep, sep)), r);
            }
            rho[i] = r;
        }
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {  // lambdas (two loops, as the reference)
            V3<R> grad{0, 0, 0};
            for (uint32_t k = 0; k < grid.cnt[i]; ++k) {
                const int j = nb(i, k);
                const V3<R> g = K.spiky(sub(xs[i], xs[j]));
                grad = {fmac<FMA>(m[j], g.x, grad.x), fmac<FMA>(m[j], g.y, grad.y),
                        fmac<FMA>(m[j], g.z, grad.z)};
            }
            grad = {grad.x * inv_rho0, grad.y * inv_rho0, grad.z * inv_rho0};
            R sum = 0;
            for (uint32_t k = 0; k < grid.cnt[i]; ++k) {
                const int j = nb(i, k);
                const V3<R> g = K.spiky(sub(xs[i], xs[j]));
                const R s = (-inv_rho0) * m[j];
                const V3<R> gj{s * g.x, s * g.y, s * g.z};
                sum = sum + dot3<FMA>(gj, gj);
            }
            const R c = fmac<FMA>(rho[i], inv_rho0, R(-1));
            lam[i] = (-c) / ((sum + dot3<FMA>(grad, grad)) + relax);
        }
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {  // position deltas with artificial pressure
            V3<R> d{0, 0, 0};
            for (uint32_t k = 0; k < grid.cnt[i]; ++k) {
                const int j = nb(i, k);
                const V3<R> sep = sub(xs[i], xs[j]);
                const R ratio = K.poly6(dot3<FMA>(sep, sep)) / wdq;
                const R pw = n_int ? pown(ratio, n_i) : (R)std::pow(ratio, (R)P.corr_n);
                // lambda_corr = -k * pw is a product used once as an addend: contracted into
                // (lambda_i + lambda_j) + lambda_corr like every a*b + c of the reference
                const R b = fmac<FMA>(neg_k, pw, lam[i] + lam[j]) * m[j];
                const V3<R> g = K.spiky(sep);
                d = {fmac<FMA>(b, g.x, d.x), fmac<FMA>(b, g.y, d.y), fmac<FMA>(b, g.z, d.z)};
            }
            dp[i] = {d.x * inv_rho0, d.y * inv_rho0, d.z * inv_rho0};
        }
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {  // correct + soft box clamp
            V3<R> p{xs[i].x + dp[i].x, xs[i].y + dp[i].y, xs[i].z + dp[i].z};
            R* pc = &p.x;
            for (int a = 0; a < 3; ++a) {
                const R lo = (R)P.box_min[a] + md, hi = (R)P.box_max[a] - md;
                R c = 0;
                if (pc[a] < lo) c = fmac<FMA>(stiff, lo - pc[a], c);
                if (pc[a] > hi) c = fmac<FMA>(stiff, hi - pc[a], c);
                pc[a] = pc[a] + c;
            }
            for (int k = 0; k < P.num_shapes; ++k) {  // SDF obstacles
                R g[3];
                const R phi = sdf_eval<R>(P.shapes[k], p.x, p.y, p.z, g);
                if (phi < (R)P.sdf_min_dist) {
                    const R c = (R)P.sdf_stiffness * ((R)P.sdf_min_dist - phi);
                    p = {p.x + c * g[0], p.y + c * g[1], p.z + c * g[2]};
                }
            }
            xs_next[i] = p;
        }
        std::swap(xs, xs_next);
    }

    // 6. update (kernel_update_position_and_velocity)
    const R rdt = (R)dt;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        vstar[i] = {(xs[i].x - x[i].x) / rdt, (xs[i].y - x[i].y) / rdt, (xs[i].z - x[i].z) / rdt};
        x[i] = xs[i];
        v[i] = vstar[i];
    }
    // 7. boundary velocity damping (resolve_collision over six planes)
    const R rest = (R)P.restitution;
    const R keep = fp64 ? (R)(1.0 - (double)P.friction) : (R)(1.0f - P.friction);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const V3<R> pts[6] = {{(R)P.box_min[0], 0, 0}, {(R)P.box_max[0], 0, 0},
                              {0, (R)P.box_min[1], 0}, {0, (R)P.box_max[1], 0},
                              {0, 0, (R)P.box_min[2]}, {0, 0, (R)P.box_max[2]}};
        const V3<R> nrm[6] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        V3<R> vel = v[i];
        for (int q = 0; q < 6; ++q) {
            const R dist = dot3<FMA>(sub(x[i], pts[q]), nrm[q]);
            const R appr = dot3<FMA>(vel, nrm[q]);
            if (dist < md) {
                const V3<R> vn{appr * nrm[q].x, appr * nrm[q].y, appr * nrm[q].z};
                const V3<R> vt = sub(vel, vn);
                if (appr < R(0)) {
                    vel = {fmac<FMA>(-rest, vn.x, keep * vt.x), fmac<FMA>(-rest, vn.y, keep * vt.y),
                           fmac<FMA>(-rest, vn.z, keep * vt.z)};
                } else if (std::fabs(appr) < (R)1e-5f) {
                    vel = {keep * vt.x, keep * vt.y, keep * vt.z};
                }
            }
        }
        for (int k = 0; k < P.num_shapes; ++k) {  // SDF obstacles, plain dot products
            R g[3];
            const R dist = sdf_eval<R>(P.shapes[k], x[i].x, x[i].y, x[i].z, g);
            const R appr = vel.x * g[0] + vel.y * g[1] + vel.z * g[2];
            if (dist < (R)P.sdf_min_dist) {
                const V3<R> vn{appr * g[0], appr * g[1], appr * g[2]};
                const V3<R> vt = sub(vel, vn);
                if (appr < R(0)) {
                    vel = {fmac<FMA>(-rest, vn.x, keep * vt.x), fmac<FMA>(-rest, vn.y, keep * vt.y),
                           fmac<FMA>(-rest, vn.z, keep * vt.z)};
                } else if (std::fabs(appr) < (R)1e-5f) {
                    vel = {keep * vt.x, keep * vt.y, keep * vt.z};
                }
            }
        }
        v[i] = vel;
    }
    // 8. vorticity
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        V3<R> w{0, 0, 0};
        for (uint32_t k = 0; k < grid.cnt[i]; ++k) {
            const int j = nb(i, k);
            const V3<R> vij = sub(v[j], v[i]);
            const V3<R> g = K.spiky(sub(x[i], x[j]));
            const V3<R> c = cross3<FMA>(vij, g);
            const R s = -m[j];
            w = {fmac<FMA>(s, c.x, w.x), fmac<FMA>(s, c.y, w.y), fmac<FMA>(s, c.z, w.z)};
        }
        omega[i] = w;
    }
    // 9. vorticity confinement (writes only the particle's own velocity)
    std::vector<R> wlen(n);
    for (int i = 0; i < n; ++i) wlen[i] = std::sqrt(dot3<FMA>(omega[i], omega[i]));
    const R veps = (R)P.vorticity_epsilon;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const R inv_d = R(1) / rho[i];
        V3<R> eta{0, 0, 0};
        for (uint32_t k = 0; k < grid.cnt[i]; ++k) {
            const int j = nb(i, k);
            const R s = m[j] * (wlen[i] - wlen[j]);
            const V3<R> g = K.spiky(sub(x[i], x[j]));
            eta = {fmac<FMA>(s, g.x, eta.x), fmac<FMA>(s, g.y, eta.y), fmac<FMA>(s, g.z, eta.z)};
        }
        eta = {eta.x * inv_d, eta.y * inv_d, eta.z * inv_d};
        const R len = std::sqrt(dot3<FMA>(eta, eta));
        if (len < (R)1e-5f) continue;
        const V3<R> N{eta.x / len, eta.y / len, eta.z / len};
        const V3<R> c = cross3<FMA>(N, omega[i]);
        const V3<R> f{veps * c.x, veps * c.y, veps * c.z};
        v[i] = {fmac<FMA>(rdt, f.x, v[i].x), fmac<FMA>(rdt, f.y, v[i].y), fmac<FMA>(rdt, f.z, v[i].z)};
    }
    // 10. XSPH viscosity from a snapshot of the post-confinement velocities
    const std::vector<V3<R>> vsnap = v;
    const R cx = (R)P.viscosity;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        V3<R> vd{0, 0, 0};
        for (uint32_t k = 0; k < grid.cnt[i]; ++k) {
            const int j = nb(i, k);
            const V3<R> vij = sub(vsnap[j], vsnap[i]);
            const V3<R> sep = sub(x[i], x[j]);
            const R w = K.poly6(dot3<FMA>(sep, sep));
            const R s = m[j] / rho[j];
            const V3<R> t{s * vij.x, s * vij.y, s * vij.z};
            vd = {fmac<FMA>(t.x, w, vd.x), fmac<FMA>(t.y, w, vd.y), fmac<FMA>(t.z, w, vd.z)};
        }
        v[i] = {fmac<FMA>(cx, vd.x, vsnap[i].x), fmac<FMA>(cx, vd.y, vsnap[i].y),
                fmac<FMA>(cx, vd.z, vsnap[i].z)};
    }
    // 11. write the records back in sorted order (the reference sorts the buffer in place)
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        ParticleRec& p = ps[i];
        for (int a = 0; a < 3; ++a) {
            p.position[a] = (float)(&x[i].x)[a];
            p.velocity[a] = (float)(&v[i].x)[a];
            p.new_position[a] = (float)(&x[i].x)[a];
            p.new_velocity[a] = (float)(&vstar[i].x)[a];
            p.position_delta[a] = (float)(&dp[i].x)[a];
            p.vorticity[a] = (float)(&omega[i].x)[a];
        }
        p.density = (float)rho[i];
        p.lambda = (float)lam[i];
    }
    std::memcpy(particles, ps.data(), sizeof(ParticleRec) * n);
    return 0;
}

}  // namespace

extern "C" {

int oracle_abi_version(void) { return 1; }
int oracle_particle_size(void) { return (int)sizeof(ParticleRec); }

// One PBFSolver::step over `n` records in the reference Particle layout, in place.  Optional
// outputs: perm[s] = pre-sort index of the record now at slot s; nbr (n*max_neighbours, row-major)
// and cnt = the neighbour lists of the sorted particles.
int oracle_step(const OracleParams* P, int n, void* particles, uint32_t* perm, uint32_t* nbr,
                uint32_t* cnt) {
    if (!P || n < 0 || (n > 0 && !particles)) return -1;
    if (P->max_neighbours <= 0 || P->table_size <= 0 || P->solver_iterations < 0) return -1;
    if (n == 0) return 0;
#ifdef _OPENMP
    if (P->num_threads > 0) omp_set_num_threads(P->num_threads);
#endif
    ParticleRec* ps = static_cast<ParticleRec*>(particles);
    const bool fma = (P->flags & ORACLE_FMA) != 0;
    const bool fp64 = (P->flags & ORACLE_FP64) != 0;
    if (fma && fp64) return step_impl<true, double>(*P, n, ps, perm, nbr, cnt);
    if (fma) return step_impl<true, float>(*P, n, ps, perm, nbr, cnt);
    if (fp64) return step_impl<false, double>(*P, n, ps, perm, nbr, cnt);
    return step_impl<false, float>(*P, n, ps, perm, nbr, cnt);
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Known-answer helpers.
float oracle_poly6(float r2, float h) { return make_kernels<true, float>(h).poly6(r2); }
void oracle_spiky(const float* rv, float h, float* out) {
    V3<float> g = make_kernels<true, float>(h).spiky(V3<float>{rv[0], rv[1], rv[2]});
    out[0] = g.x; out[1] = g.y; out[2] = g.z;
}
uint32_t oracle_hash(int cx, int cy, int cz, int32_t table) { return cell_hash(cx, cy, cz, (uint32_t)table); }
int oracle_cell(float x, float cell) { return cell_coord(x, cell); }

}  // extern "C"
